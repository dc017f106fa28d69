"""Batched execution (one CUDA graph: persistent work queue + standalone
partitioned launches) gives every instance exactly its per-instance result."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mix(bale, oracle, cuda, seed: int, big: bool):
    import torch

    from bale_old_gb300 import batch

    rng = np.random.default_rng(seed)
    insts, checks = [], []
    logu = lambda lo, hi: int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))  # noqa: E731
    # histograms: tables on both sides of the shared-memory limit, some packed,
    # some with out-of-range updates
    for k in range(40):
        t = [1, 7, 977, 48 * 1024, 48 * 1024 + 1][k % 5] if k < 10 else logu(2, 1 << 21)
        n = logu(1, 1 << 20)
        idx = bale.gen_uniform(n, t + (t // 50 if k % 7 == 3 else 0), 100 * seed + k)
        shift = 16 if k % 4 == 1 else 0
        counts0 = bale.gen_uniform(t, 5, k)
        ok = idx < t
        want = counts0 + np.bincount(idx[ok], minlength=t)
        d_idx = torch.from_numpy(bale.pack_index(idx) if shift else idx).to(cuda)
        d_cnt = torch.from_numpy(counts0).to(cuda)
        insts.append(batch.histo(d_cnt, d_idx, shift=shift))
        checks.append(("histo", d_cnt, want, int((~ok).sum())))
    for k in range(30):
        t = logu(1, 1 << 22)
        n = logu(1, 1 << 20)
        idx = bale.gen_uniform(n, t + (5 if k % 6 == 2 else 0), 200 * seed + k)
        table = bale.gen_values(t, k + 7)
        ok = idx < t
        want = np.where(ok, table[np.minimum(idx, t - 1)], 0)
        d_tgt = torch.full((n,), 99, dtype=torch.int64, device=cuda)
        insts.append(batch.ig(d_tgt, torch.from_numpy(idx).to(cuda), torch.from_numpy(table).to(cuda)))
        checks.append(("ig", d_tgt, want, int((~ok).sum())))
    for k, scale in enumerate((4, 6, 8, 9, 10, 11, 12, 13)):
        L = bale.gen_rmat(scale, 16, 0.57, 0.19, 0.19, 300 * seed + k)
        want = oracle.triangle_agi(L.offset, L.nonzero)[0]
        d_cnt = torch.zeros(1, dtype=torch.int64, device=cuda)
        insts.append(batch.triangles(torch.from_numpy(L.offset).to(cuda), torch.from_numpy(L.nonzero).to(cuda), d_cnt))
        checks.append(("tri", d_cnt, want, 0))
    if big:  # big enough for the standalone region-partitioned kernels
        t, n = (1 << 24) + 3, (1 << 20) + 5
        idx = bale.gen_uniform(n, t, 11 + seed)
        table = bale.gen_values(t, 12)
        d_tgt = torch.empty(n, dtype=torch.int64, device=cuda)
        insts.append(batch.ig(d_tgt, torch.from_numpy(idx).to(cuda), torch.from_numpy(table).to(cuda)))
        checks.append(("ig", d_tgt, table[idx], 0))
        idx = bale.gen_uniform(n, 1 << 24, 13 + seed)
        d_cnt = torch.zeros(1 << 24, dtype=torch.int64, device=cuda)
        insts.append(batch.histo(d_cnt, torch.from_numpy(idx).to(cuda)))
        checks.append(("histo", d_cnt, np.bincount(idx, minlength=1 << 24), 0))
        L = bale.gen_rmat(18, 16, 0.57, 0.19, 0.19, 14 + seed)  # > 2^21 nonzeros: its own kernels
        d_cnt = torch.zeros(1, dtype=torch.int64, device=cuda)
        insts.append(batch.triangles(torch.from_numpy(L.offset).to(cuda), torch.from_numpy(L.nonzero).to(cuda), d_cnt))
        checks.append(("tri", d_cnt, oracle.triangle_agi_mt(L.offset, L.nonzero), 0))
    return insts, checks


class pinned:
    """Set tuning knobs for a block and restore their previous values."""

    def __init__(self, bale, **knobs):
        self.bale, self.knobs = bale, {k.replace("__", "."): v for k, v in knobs.items()}

    def __enter__(self):
        self.old = {k: self.bale.tune_get(k) for k in self.knobs}
        for k, v in self.knobs.items():
            self.bale.tune_set(k, v)

    def __exit__(self, *exc):
        for k, v in self.old.items():
            self.bale.tune_set(k, v)


# the standalone thresholds the assertions below count against
DEFAULT_RULES = dict(ig__part_min_table_bytes=96 << 20, ig__part_min_requests=1 << 20,
                     histo__part_min_table_bytes=96 << 20, histo__part_min_updates=1 << 20,
                     batch__standalone_min=1 << 23, batch__standalone_min_edges=1 << 21)


@pytest.mark.parametrize("standalone", [-1, 0])
def test_mixed_batch_matches_per_instance_results(cuda, bale, oracle, standalone):
    import torch

    from bale_old_gb300 import batch

    with pinned(bale, batch__standalone=standalone, **DEFAULT_RULES):
        insts, checks = _mix(bale, oracle, cuda, seed=1, big=True)
        starts = [c[1].clone() for c in checks]
        with batch.Batch(insts) as b:
            st = b.stats()
            assert st["instances"] == len(insts)
            if standalone == 0:
                assert st["standalone_instances"] == 0
            else:
                assert st["standalone_instances"] == 3
            b.run()
            b.run()  # replaying the graph: histo/triangles accumulate, ig overwrites
            torch.cuda.synchronize()
            bad = b.bad()
        for k, (kind, dev, want, nbad) in enumerate(checks):
            got = dev.cpu().numpy()
            if kind == "histo":
                start = starts[k].cpu().numpy()
                np.testing.assert_array_equal(got, start + 2 * (want - start), err_msg=f"histo {k}")
            elif kind == "ig":
                np.testing.assert_array_equal(got, want, err_msg=f"ig {k}")
            else:
                assert int(got[0]) == 2 * want, (k, int(got[0]), want)
            assert bad[k] == nbad, (k, kind, int(bad[k]), nbad)


def test_many_standalone_instances_on_several_streams(cuda, bale, oracle):
    """Low standalone thresholds: most instances run their own kernels,
    spread over the side streams of the graph, concurrently with the queue."""
    import torch

    from bale_old_gb300 import batch

    with pinned(bale, batch__standalone_min=1000, batch__standalone_min_edges=1000, batch__streams=3):
        insts, checks = _mix(bale, oracle, cuda, seed=3, big=True)
        starts = [c[1].clone() for c in checks]
        with batch.Batch(insts) as b:
            st = b.stats()
            assert st["standalone_instances"] > 40 and st["side_streams"] == 3
            b.run()
            torch.cuda.synchronize()
            bad = b.bad()
        for k, (kind, dev, want, nbad) in enumerate(checks):
            got = dev.cpu().numpy()
            if kind == "tri":
                assert int(got[0]) == want
            else:
                np.testing.assert_array_equal(got, want, err_msg=f"{kind} {k}")
            assert bad[k] == nbad, (k, kind)
        del starts


def test_tiny_tiles_and_knobs_do_not_change_results(cuda, bale, oracle):
    import torch

    from bale_old_gb300 import batch

    names = {f"batch__{b}__{c}": (1 if "rows" in b else 1000)
             for b in ("histo_tile", "histo_l2_tile", "ig_tile", "tri_heavy_rows", "tri_light_rows")
             for c in ("small", "medium", "large")}
    with pinned(bale, **names):
        insts, checks = _mix(bale, oracle, cuda, seed=2, big=False)
        starts = [c[1].clone() for c in checks]
        with batch.Batch(insts) as b:
            b.run()
            torch.cuda.synchronize()
        for k, (kind, dev, want, nbad) in enumerate(checks):
            got = dev.cpu().numpy()
            if kind == "histo":
                np.testing.assert_array_equal(got, want, err_msg=f"histo {k}")
            elif kind == "ig":
                np.testing.assert_array_equal(got, want, err_msg=f"ig {k}")
            else:
                assert int(got[0]) == want
        del starts


def test_empty_and_degenerate_batches(cuda, bale):
    import torch

    from bale_old_gb300 import batch

    with batch.Batch([]) as b:
        b.run()
        torch.cuda.synchronize()
        assert b.stats()["tasks"] == 0
    z = torch.zeros(0, dtype=torch.int64, device=cuda)
    c = torch.zeros(4, dtype=torch.int64, device=cuda)
    one = torch.zeros(1, dtype=torch.int64, device=cuda)
    off = torch.zeros(1, dtype=torch.int64, device=cuda)
    with batch.Batch([batch.histo(c, z), batch.ig(z, z, c), batch.triangles(off, z, one)]) as b:
        b.run()
        torch.cuda.synchronize()
        assert not c.any() and int(one.item()) == 0


def test_invalid_instance_is_rejected(cuda, bale):
    import torch

    from bale_old_gb300 import batch

    c = torch.zeros(4, dtype=torch.int64, device=cuda)
    bad = batch.Instance(7, 0, 4, 4, c, c, None)
    with pytest.raises(bale.BaleError):
        batch.Batch([bad])


def test_device_generators_match_host_generators(cuda, bale):
    import torch

    for n, rng, seed, packed in ((1, 1, 0, False), (1000, 77, 5, True), (1 << 20, (1 << 26) + 3, 9, False)):
        d = torch.empty(n, dtype=torch.int64, device=cuda)
        bale.gen_uniform_dev(d, rng, seed, packed)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(d.cpu().numpy(), bale.gen_uniform(n, rng, seed, packed))
    d = torch.empty(12345, dtype=torch.int64, device=cuda)
    bale.gen_values_dev(d, 17)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d.cpu().numpy(), bale.gen_values(12345, 17))
