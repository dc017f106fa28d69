"""Histogram on the GPU, through the C ABI, bit-exact against the oracle and
the reference's golden vectors.  Table sizes cover every kernel path: the
shared-memory private table, warp-aggregated L2 reductions and plain ones."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_golden_vectors_accumulate_across_models(cuda, bale, golden):
    """The reference app runs agi, exstack, exstack2 into one counts array
    (apps/histo_src/histo.upc:161-213); the drop-ins must ADD the same way."""
    d = golden("histo")
    for name in sorted({k.split("/")[0] for k in d.files}):
        index = d[f"{name}/index"]
        pck = bale.pack_index(index)
        c = d[f"{name}/counts0"].copy()
        bale.histo_agi(index, c)
        np.testing.assert_array_equal(c, d[f"{name}/after_agi"], err_msg=name)
        bale.histo_exstack(pck, c)
        np.testing.assert_array_equal(c, d[f"{name}/after_exstack"], err_msg=name)
        bale.histo_exstack2(pck, c)
        np.testing.assert_array_equal(c, d[f"{name}/after_exstack2"], err_msg=name)
        bale.histo_conveyor(pck, c)  # a fourth model adds once more
        want = d[f"{name}/after_exstack2"] + np.bincount(index, minlength=c.size)
        np.testing.assert_array_equal(c, want, err_msg=name)


@pytest.mark.parametrize("n,tsize", [(0, 10), (1, 1), (3, 2), (1000, 1), (100_000, 1_000),
                                     (300_001, 48 * 1024), (300_001, 48 * 1024 + 1),
                                     (1 << 20, 1 << 20), (1 << 20, (1 << 20) + 1),
                                     (2_000_000, 1 << 23)])
def test_random_sizes_match_oracle(cuda, bale, oracle, n, tsize):
    index = bale.gen_uniform(n, tsize, 7 * n + tsize) if n else np.zeros(0, np.int64)
    counts = bale.gen_uniform(tsize, 50, 11)
    want = counts.copy()
    oracle.histo_agi(index, want)
    bale.histo_agi(index, counts)
    np.testing.assert_array_equal(counts, want)


@pytest.mark.parametrize("tsize", [1, 64, 5_000, 1 << 20, 1 << 22])
def test_heavy_collisions(cuda, bale, oracle, tsize):
    """All-same and Zipf-skewed updates: warp aggregation must merge exactly."""
    same = np.full(100_001, tsize - 1, np.int64)
    c = np.zeros(tsize, np.int64)
    bale.histo_agi(same, c)
    assert c[tsize - 1] == same.size and c.sum() == same.size
    z = bale.gen_zipf(500_000, tsize, 1.1, 1, 2) if tsize > 1 else np.zeros(500_000, np.int64)
    c = np.zeros(tsize, np.int64)
    want = c.copy()
    oracle.histo_agi(z, want)
    bale.histo_agi(z, c)
    np.testing.assert_array_equal(c, want)


def test_unaligned_index(cuda, bale, oracle):
    base = bale.gen_uniform(50_001, 3_000, 4)
    index = base[1:]
    for tsize in (3_000, 1 << 20):
        c = np.zeros(tsize, np.int64)
        want = c.copy()
        oracle.histo_agi(np.ascontiguousarray(index), want)
        bale.histo_agi(index, c)
        np.testing.assert_array_equal(c, want)


def test_out_of_range_is_an_error_not_a_fault(cuda, bale):
    c = np.zeros(10, np.int64)
    with pytest.raises(bale.BaleError):
        bale.histo_agi(np.array([1, -2, 3], np.int64), c)
    bale.histo_agi(np.array([1, 1, 3], np.int64), c)
    assert c[1] == 2 and c[3] == 1


def test_device_entry_point_and_bad_counter(cuda, bale):
    import torch

    for tsize in (100, 100_000, 1 << 21):
        idx_h = bale.gen_uniform(200_000, tsize + tsize // 10 + 1, tsize)
        idx = torch.from_numpy(idx_h).to(cuda)
        counts = torch.zeros(tsize, dtype=torch.int64, device=cuda)
        bad = torch.zeros(1, dtype=torch.int64, device=cuda)
        bale.histo_dev(counts, idx, bad=bad)
        torch.cuda.synchronize()
        ok = idx_h < tsize
        assert int(bad.item()) == int((~ok).sum())
        np.testing.assert_array_equal(counts.cpu().numpy(), np.bincount(idx_h[ok], minlength=tsize))


def test_full_size_config_1e7_updates_1e6_counters(cuda, bale, oracle):
    index = bale.gen_uniform(10_000_000, 1_000_000, 1)
    c = np.zeros(1_000_000, np.int64)
    bale.histo_agi(index, c)
    np.testing.assert_array_equal(c, np.bincount(index, minlength=1_000_000))
    # the reference's self-check: subtract num_models per update -> all zero
    bale.histo_exstack(bale.pack_index(index), c)
    np.subtract.at(c, index, 2)
    assert not c.any()


@pytest.mark.parametrize("hmode", [0, 1, 2, 3])
@pytest.mark.parametrize("n,tsize", [(1, 1), (3_001, 977), (100_003, 48 * 1024),
                                     (300_001, (1 << 22) + 5), (2_000_001, 3 * (1 << 22) + 1)])
def test_every_mode_matches_oracle(cuda, bale, oracle, hmode, n, tsize):
    """histo.mode 0..3 give identical counts (modes that cannot serve a size
    fall back to one that can), including invalid updates."""
    bale.tune_set("histo.mode", hmode)
    try:
        index = bale.gen_uniform(n, tsize, n + 3 * tsize)
        counts = bale.gen_uniform(tsize, 9, 5)
        want = counts.copy()
        oracle.histo_agi(index, want)
        bale.histo_agi(index, counts)
        np.testing.assert_array_equal(counts, want)
        oracle.histo_agi(index, want)
        bale.histo_exstack(bale.pack_index(index), counts)  # packed indices (>> 16)
        np.testing.assert_array_equal(counts, want)
        import torch
        idx_h = index.copy()
        idx_h[::101] = tsize + 7  # out of range
        idx = torch.from_numpy(idx_h).to(cuda)
        c = torch.zeros(tsize, dtype=torch.int64, device=cuda)
        bad = torch.zeros(1, dtype=torch.int64, device=cuda)
        bale.histo_dev(c, idx, bad=bad)
        torch.cuda.synchronize()
        ok = idx_h < tsize
        assert int(bad.item()) == int((~ok).sum())
        np.testing.assert_array_equal(c.cpu().numpy(), np.bincount(idx_h[ok], minlength=tsize))
    finally:
        bale.tune_set("histo.mode", -1)


def test_l2_reduction_probe_adds_exactly_n(cuda, bale):
    """The roofline probe lands every one of its n reductions inside the table."""
    import torch

    counts = torch.zeros(1_000_003, dtype=torch.int64, device=cuda)
    bale.l2_red_rate(counts, 12_345_678)
    torch.cuda.synchronize()
    assert int(counts.sum().item()) == 12_345_678 and int(counts.min().item()) >= 0
