"""Index gather on the GPU, through the C ABI, bit-exact against the oracle
and the reference's golden vectors."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DROPINS_PACKED = ("ig_exstack", "ig_exstack2", "ig_conveyor")


def test_golden_vectors_all_dropins(cuda, bale, golden):
    d = golden("ig")
    for name in sorted({k.split("/")[0] for k in d.files}):
        index, table, want = d[f"{name}/index"], d[f"{name}/table"], d[f"{name}/tgt"]
        tgt = np.full(index.size, 12345, np.int64)
        bale.ig_agi(tgt, index, table)
        np.testing.assert_array_equal(tgt, want, err_msg=name)
        pck = bale.pack_index(index)
        for fn in DROPINS_PACKED:
            tgt[:] = 0
            getattr(bale, fn)(tgt, pck, table)
            np.testing.assert_array_equal(tgt, want, err_msg=f"{name}/{fn}")


@pytest.mark.parametrize("n,tsize", [(0, 5), (1, 1), (2, 3), (3, 7), (31, 1000), (1000, 1),
                                     (65_537, 4_096), ((1 << 20) + 3, 1 << 20), (1 << 21, 1 << 24)])
def test_random_sizes_match_oracle(cuda, bale, oracle, n, tsize):
    index = bale.gen_uniform(n, tsize, n + tsize) if n else np.zeros(0, np.int64)
    table = bale.gen_values(tsize, 3 * tsize + 1)
    tgt = np.zeros(n, np.int64)
    bale.ig_agi(tgt, index, table)
    np.testing.assert_array_equal(tgt, oracle.ig_agi(index, table))


def test_zipf_and_negative_table_self_check(cuda, bale, oracle):
    index = bale.gen_zipf(1 << 20, 1 << 22, 1.1, 4, 5)
    table = bale.gen_negative_table(1 << 22)
    tgt = np.zeros(index.size, np.int64)
    bale.ig_agi(tgt, index, table)
    np.testing.assert_array_equal(tgt, -(index + 1))  # apps/ig_src/ig.upc:96-114


def test_unaligned_buffers_take_the_scalar_path(cuda, bale, oracle):
    base = bale.gen_uniform(10_001, 5_000, 9)
    index = base[1:]  # 8-byte but not 16-byte aligned
    table = bale.gen_values(5_000, 10)
    out = np.zeros(10_001, np.int64)
    tgt = out[1:]
    bale.ig_agi(tgt, index, table)
    np.testing.assert_array_equal(tgt, oracle.ig_agi(np.ascontiguousarray(index), table))


def test_out_of_range_index_is_an_error_not_a_fault(cuda, bale):
    table = bale.gen_values(100, 1)
    tgt = np.zeros(4, np.int64)
    with pytest.raises(bale.BaleError):
        bale.ig_agi(tgt, np.array([1, 2, -3, 4], np.int64), table)
    # the library stays usable afterwards
    bale.ig_agi(tgt, np.array([1, 2, 3, 4], np.int64), table)
    np.testing.assert_array_equal(tgt, table[[1, 2, 3, 4]])


def test_device_entry_point_counts_bad_indices(cuda, bale, oracle):
    import torch

    table_h = bale.gen_values(1000, 4)
    index_h = bale.gen_uniform(5000, 1200, 5)  # some beyond the 1000-entry table
    table, index = torch.from_numpy(table_h).to(cuda), torch.from_numpy(index_h).to(cuda)
    tgt = torch.empty_like(index)
    bad = torch.zeros(1, dtype=torch.int64, device=cuda)
    bale.ig_dev(tgt, index, table, bad=bad)
    torch.cuda.synchronize()
    ok = index_h < 1000
    assert int(bad.item()) == int((~ok).sum())
    got = tgt.cpu().numpy()
    np.testing.assert_array_equal(got[ok], table_h[index_h[ok]])
    assert not got[~ok].any()


def test_full_size_property_2e28_requests(cuda, bale):
    """2^26-entry table, 2^28 requests: table[i] = -(i+1) makes every output
    -(index+1), checked on the device (size-independent self-check)."""
    import torch

    tsize, n = 1 << 26, 1 << 28
    table = -(torch.arange(tsize, dtype=torch.int64, device=cuda) + 1)
    g = torch.Generator(device=cuda).manual_seed(3)
    index = torch.randint(0, tsize, (n,), dtype=torch.int64, device=cuda, generator=g)
    tgt = torch.empty_like(index)
    bad = torch.zeros(1, dtype=torch.int64, device=cuda)
    bale.ig_dev(tgt, index, table, bad=bad)
    torch.cuda.synchronize()
    assert int(bad.item()) == 0
    assert bool(torch.equal(tgt, -(index + 1)))
    del table, index, tgt
    torch.cuda.empty_cache()


@pytest.mark.parametrize("mode", [-1, 1], ids=["default", "partitioned"])
def test_full_size_zipf_property_2e28_requests(cuda, bale, mode):
    """The skewed ig configuration at its own size: 2^28 requests drawn
    Zipf(1.1) over a keyed permutation of a 2^26-entry table whose entries
    are table[i] = -(i+1), so every output must be -(index+1) (the check of
    apps/ig_src/ig.upc:96-114), compared in full on the device.  The default
    path sends this stream to the direct gather (the skew test); ig.mode 1
    forces the region-partitioned gather on the same data."""
    import torch

    tsize, n = 1 << 26, 1 << 28
    index = torch.from_numpy(bale.gen_zipf(n, tsize, 1.1, 4, 5)).to(cuda)
    table = -(torch.arange(tsize, dtype=torch.int64, device=cuda) + 1)
    tgt = torch.zeros_like(index)
    bad = torch.zeros(1, dtype=torch.int64, device=cuda)
    bale.tune_set("ig.mode", mode)
    try:
        bale.ig_dev(tgt, index, table, bad=bad)
        torch.cuda.synchronize()
    finally:
        bale.tune_set("ig.mode", -1)
    assert int(bad.item()) == 0
    assert bool(torch.equal(tgt, -(index + 1)))
    del table, index, tgt
    torch.cuda.empty_cache()


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("n,tsize", [(1, 1), (1000, 7), (1024, 1 << 22), (1025, (1 << 22) + 1),
                                     (5 * 1024 + 17, 3 * (1 << 22) + 5), (300_001, 1 << 24)])
def test_both_gather_modes_match_oracle(cuda, bale, oracle, mode, n, tsize):
    """ig.mode 0 (direct) and 1 (region-partitioned) give identical bits,
    including partial chunks, partial regions and single-entry tables."""
    bale.tune_set("ig.mode", mode)
    try:
        index = bale.gen_uniform(n, tsize, n ^ tsize)
        table = bale.gen_values(tsize, tsize + 17)
        tgt = np.zeros(n, np.int64)
        bale.ig_agi(tgt, index, table)
        np.testing.assert_array_equal(tgt, oracle.ig_agi(index, table))
        pck = bale.pack_index(index)
        tgt[:] = -1
        bale.ig_exstack(tgt, pck, table)
        np.testing.assert_array_equal(tgt, oracle.ig_agi(index, table))
    finally:
        bale.tune_set("ig.mode", -1)


@pytest.mark.parametrize("regions", [32, 61, 62, 63])
@pytest.mark.parametrize("shift", [0, 16])
def test_partitioned_gather_region_counts_around_the_warp_scan(cuda, bale, regions, shift):
    """The whole-chunk partition scans its region counters with one warp when
    the regions plus the out-of-range bucket and the total fit 64 slots, and
    with the block scan beyond: tables of 32, 61, 62 and 63 16-MiB regions
    (the last one partial), 2^20 + 5 requests with some out of range, plain
    and packed (>> 16) indices; table[i] = -(i+1), checked on the device."""
    import torch

    tsize = ((regions - 1) << 21) + 12345
    n = (1 << 20) + 5
    idx = bale.gen_uniform(n, tsize + 3000, regions + shift)
    idx[::1777] = -3
    table = -(torch.arange(tsize, dtype=torch.int64, device=cuda) + 1)
    index = torch.from_numpy(bale.pack_index(idx) if shift else idx).to(cuda)
    want_idx = torch.from_numpy(idx).to(cuda)
    ok = (want_idx >= 0) & (want_idx < tsize)
    tgt = torch.full_like(index, 7)
    bad = torch.zeros(1, dtype=torch.int64, device=cuda)
    bale.tune_set("ig.mode", 1)
    try:
        bale.ig_dev(tgt, index, table, shift=shift, bad=bad)
        torch.cuda.synchronize()
    finally:
        bale.tune_set("ig.mode", -1)
    assert int(bad.item()) == int((~ok).sum().item())
    assert bool(torch.equal(tgt, torch.where(ok, -(want_idx + 1), torch.zeros_like(want_idx))))
    del table, index, tgt
    torch.cuda.empty_cache()


@pytest.mark.parametrize("mode", [0, 1])
def test_both_modes_count_bad_indices(cuda, bale, mode):
    import torch

    bale.tune_set("ig.mode", mode)
    try:
        tsize = (1 << 22) + 3
        table_h = bale.gen_values(tsize, 8)
        index_h = bale.gen_uniform(70_001, tsize + 5000, 9)
        index_h[::1000] = -5
        table, index = torch.from_numpy(table_h).to(cuda), torch.from_numpy(index_h).to(cuda)
        tgt = torch.empty_like(index)
        bad = torch.zeros(1, dtype=torch.int64, device=cuda)
        bale.ig_dev(tgt, index, table, bad=bad)
        torch.cuda.synchronize()
        ok = (index_h >= 0) & (index_h < tsize)
        assert int(bad.item()) == int((~ok).sum())
        got = tgt.cpu().numpy()
        np.testing.assert_array_equal(got[ok], table_h[index_h[ok]])
        assert not got[~ok].any()
    finally:
        bale.tune_set("ig.mode", -1)


@pytest.fixture
def small_chunks(bale):
    """Pipelined drop-in with 4096-request chunks, so small calls take it."""
    bale.tune_set("dropin.ig_chunk", 4096)
    yield 4096
    bale.tune_set("dropin.ig_chunk", -1)


@pytest.mark.parametrize("order", ["uniform", "ascending", "late_max", "packed"])
def test_pipelined_dropin_matches_oracle(cuda, bale, oracle, small_chunks, order):
    """Chunked uploads, per-chunk maxima and overlapped gathers and downloads
    give the single-pass result.  "ascending" indices make every chunk reach
    beyond the table uploaded for the first one (extension and a larger
    buffer); "late_max" puts the only large index in the last chunk."""
    n, t = 50_001, 1 << 18
    table = bale.gen_values(t, 11)
    if order == "uniform":
        idx = bale.gen_uniform(n, t, 12)
    elif order == "ascending":
        idx = np.sort(bale.gen_uniform(n, t, 13))
    else:
        idx = bale.gen_uniform(n, 1000, 14)
        idx[-3] = t - 1
    tgt = np.full(n, -7, np.int64)
    if order == "packed":
        bale.ig_exstack(tgt, bale.pack_index(idx), table)
    else:
        bale.ig_agi(tgt, idx, table)
    np.testing.assert_array_equal(tgt, table[idx])


def test_pipelined_dropin_bad_index_is_an_error(cuda, bale, small_chunks):
    n, t = 40_000, 5000
    table = bale.gen_values(t, 3)
    idx = bale.gen_uniform(n, t, 4)
    idx[-10] = -5  # a negative index in the last chunk
    with pytest.raises(bale.BaleError):
        bale.ig_agi(np.zeros(n, np.int64), idx, table)
    idx[-10] = 7
    tgt = np.zeros(n, np.int64)
    bale.ig_agi(tgt, idx, table)
    np.testing.assert_array_equal(tgt, table[idx])


# Tables beyond L2 with skewed requests: the skew test on the device picks
# the direct gather (L1-allocating table loads) or the partitioned one; both
# must give the same values and bad counts, whatever the choice and however
# its threshold is set.
@pytest.mark.parametrize("dist", ["uniform", "zipf1.01", "zipf1.3", "zipf1.3_bad"])
@pytest.mark.parametrize("pct", [-1, 0, 1, 100])
def test_skew_switch_matches_oracle(cuda, bale, oracle, dist, pct):
    import torch

    tsize, n = 1 << 24, (1 << 22) + 5
    if dist == "uniform":
        index = bale.gen_uniform(n, tsize, 41)
    else:
        index = bale.gen_zipf(n, tsize, 1.3 if dist.startswith("zipf1.3") else 1.01, 42, 43)
    if dist.endswith("_bad"):
        index[::4097] = tsize + 7  # out-of-range requests: value 0, counted
    table = bale.gen_values(tsize, 44)
    dev = torch.device("cuda:0")
    t_index, t_table = torch.from_numpy(index).to(dev), torch.from_numpy(table).to(dev)
    tgt = torch.full((n,), 99, dtype=torch.int64, device=dev)
    bad = torch.zeros(1, dtype=torch.int64, device=dev)
    bale.tune_set("ig.skew_repeat_pct", pct)
    try:
        bale.ig_dev(tgt, t_index, t_table, bad=bad)
        torch.cuda.synchronize()
    finally:
        bale.tune_set("ig.skew_repeat_pct", -1)
    ok = index < tsize
    want = np.where(ok, table[np.where(ok, index, 0)], 0)
    np.testing.assert_array_equal(tgt.cpu().numpy(), want)
    assert int(bad.item()) == int((~ok).sum())


@pytest.mark.parametrize("dist", ["uniform", "zipf1.3"])
def test_skew_switch_inside_a_captured_graph(cuda, bale, dist):
    """The skew test, both partitioned kernels' early returns and the direct
    gather are stream work only: a warmed-up call captures into a CUDA graph
    and replays with fresh inputs."""
    import torch

    tsize, n = 1 << 24, 1 << 22
    dev = torch.device("cuda:0")
    table_h = bale.gen_values(tsize, 51)
    t_table = torch.from_numpy(table_h).to(dev)
    t_index = torch.empty(n, dtype=torch.int64, device=dev)
    tgt = torch.empty(n, dtype=torch.int64, device=dev)
    s = torch.cuda.Stream()

    def fresh(seed):
        return (bale.gen_uniform(n, tsize, seed) if dist == "uniform"
                else bale.gen_zipf(n, tsize, 1.3, seed, seed + 1))

    with torch.cuda.stream(s):  # the workspace is per stream: warm up on the capture stream
        t_index.copy_(torch.from_numpy(fresh(1)))
        bale.ig_dev(tgt, t_index, t_table)
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        bale.ig_dev(tgt, t_index, t_table)
    for seed in (5, 9):
        index_h = fresh(seed)
        t_index.copy_(torch.from_numpy(index_h))
        tgt.fill_(-1)
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(tgt.cpu().numpy(), table_h[index_h])
