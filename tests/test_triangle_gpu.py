"""Triangle counting on the GPU, through the C ABI: exact int64 counts equal
to the reference's (golden vectors, Kronecker closed forms) and to the
oracle on seeded R-MAT and Erdos-Renyi graphs up to the full scale-22 size."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DROPINS = ("triangle_agi", "triangle_exstack_push", "triangle_exstack2_push",
           "triangle_convey_push", "triangle_agi_iter")


@pytest.fixture(params=[0, 1, 2], ids=["merge", "hybrid", "wedge"])
def mode(request, bale):
    """tri.mode 0: warp-per-row merge for every row; 1: bitmap/search hybrid
    over rows i; 2: wedge probes grouped at the far vertex j (what the
    default runs below 2^23 nonzeros, and above for graphs with hubs)."""
    bale.tune_set("tri.mode", request.param)
    yield request.param
    bale.tune_set("tri.mode", -1)


def test_golden_graphs_all_dropins(cuda, bale, golden, mode):
    d = golden("triangles")
    for g in d["graphs"]:
        L = bale.SparseMatrix(d[f"{g}/offset"], d[f"{g}/nonzero"])
        want = int(d[f"{g}/triangle_agi"][0])
        for fn in DROPINS:
            cnt, sr, secs = getattr(bale, fn)(L)
            assert cnt == want, (g, fn)
            assert secs >= 0
        closed = int(d[f"{g}/closed_form"][0])
        if closed >= 0:
            assert want == closed


@pytest.mark.parametrize("kmode,specs", [(1, [3, 4, 5, 9]), (2, [3, 4, 5, 9, 2]), (0, [5, 9, 4]),
                                         (1, [1, 4, 9, 16, 25]), (1, [2000, 2]), (2, [1500, 3])])
def test_kronecker_closed_forms_including_hub_rows(cuda, bale, kmode, specs, mode):
    """Star products have hub rows far longer than a warp's shared-memory slot."""
    L = bale.gen_kronecker(kmode, specs)
    cnt, _, _ = bale.triangle_agi(L)
    assert cnt == bale.kronecker_triangles(kmode, specs)


@pytest.mark.parametrize("scale", [6, 10, 14, 16])
def test_rmat_matches_oracle(cuda, bale, oracle, scale, mode):
    L = bale.gen_rmat(scale, 16, 0.57, 0.19, 0.19, 100 + scale)
    cnt, sr, _ = bale.triangle_agi(L)
    assert cnt == oracle.triangle_agi_mt(L.offset, L.nonzero)
    deg = np.diff(L.offset)
    nf = np.ones(L.nnz, bool)
    nf[L.offset[:-1][deg > 0]] = False
    pulls = int(deg[L.nonzero[nf]].sum())
    if mode == 0:
        # the merge kernel scans every row-j element: the reference's pulls
        # for every (i,j) except the first nonzero of each row
        assert sr == pulls
    elif mode == 2:
        # one probe per element of row i below j, for every (i,j) whose row j
        # is not empty: the reference's exstack pushes, less those
        rowid = np.repeat(np.arange(L.numrows), deg)
        pos = np.arange(L.nnz) - L.offset[rowid]
        assert sr == int(pos[deg[L.nonzero] > 0].sum())
    else:
        # the hybrid streams or searches the cheaper side of each (i,j)
        assert 0 < sr <= pulls + int((deg * (deg - 1) // 2).sum())


def test_erdos_renyi_matches_oracle(cuda, bale, oracle, mode):
    n = 1 << 16
    L = bale.gen_erdos_renyi(n, 32.0 / n, 7)
    assert bale.triangle_agi(L)[0] == oracle.triangle_agi_mt(L.offset, L.nonzero)


@pytest.fixture(scope="module")
def er20(bale, oracle):
    """The Erdos-Renyi variant of the triangle configuration: n = 2^20,
    p = 32/2^20 (average degree 32), lower triangle, with the multi-threaded
    oracle's count."""
    n = 1 << 20
    L = bale.gen_erdos_renyi(n, 32.0 / n, 7)
    return L, oracle.triangle_agi_mt(L.offset, L.nonzero)


@pytest.mark.parametrize("tmode", [-1, 0, 1, 2], ids=["default", "merge", "hybrid", "wedge"])
def test_erdos_renyi_2e20_degree32_config_matches_oracle(cuda, bale, er20, tmode):
    """At its own size, in the default mode (the device-side choice picks the
    hybrid for this graph) and in each forced mode, through every drop-in:
    the count equals the oracle's, as the reference's apps require of every
    model (apps/triangle_src/triangle.upc:415-420)."""
    L, want = er20
    assert L.nnz > 16_000_000 and want > 0
    bale.tune_set("tri.mode", tmode)
    try:
        for fn in DROPINS:
            assert getattr(bale, fn)(L)[0] == want, fn
    finally:
        bale.tune_set("tri.mode", -1)


def _clique(m: int):
    off = np.zeros(m + 1, np.int64)
    off[1:] = np.cumsum(np.arange(m))
    col = np.concatenate([np.arange(i, dtype=np.int64) for i in range(m)]) if m > 1 else np.zeros(0, np.int64)
    return off, col


@pytest.mark.parametrize("m", [0, 1, 2, 3, 40, 1025, 1800])
def test_cliques_long_rows_and_tiny_graphs(cuda, bale, m, mode):
    off, col = _clique(m)
    L = bale.SparseMatrix(off, col)
    assert bale.triangle_agi(L)[0] == m * (m - 1) * (m - 2) // 6


def test_malformed_matrices_are_errors_not_faults(cuda, bale, mode):
    good_off, good_col = _clique(6)
    cases = []
    c = good_col.copy(); c[-1] = 5                      # column == row (not strict)
    cases.append((good_off, c))
    c = good_col.copy(); c[-2], c[-1] = c[-1], c[-2]    # row not ascending
    cases.append((good_off, c))
    c = good_col.copy(); c[4] = -1                      # negative column
    cases.append((good_off, c))
    o = good_off.copy(); o[3] = 99                      # offset beyond nnz
    cases.append((o, good_col))
    for off, col in cases:
        with pytest.raises(bale.BaleError):
            bale.triangle_agi(bale.SparseMatrix(off, col))
    assert bale.triangle_agi(bale.SparseMatrix(good_off, good_col))[0] == 20


def test_device_entry_point(cuda, bale, oracle):
    import torch

    L = bale.gen_rmat(13, 16, 0.57, 0.19, 0.19, 5)
    off = torch.from_numpy(L.offset).to(cuda)
    col = torch.from_numpy(L.nonzero).to(cuda)
    count = torch.zeros(1, dtype=torch.int64, device=cuda)
    bale.triangle_dev(off, col, count)
    bale.triangle_dev(off, col, count)  # accumulates
    torch.cuda.synchronize()
    assert int(count.item()) == 2 * oracle.triangle_agi(L.offset, L.nonzero)[0]


def test_full_size_rmat_scale22(cuda, bale, oracle, mode):
    """The R-MAT scale-22 configuration, exact against the multi-threaded oracle."""
    L = bale.gen_rmat(22, 16, 0.57, 0.19, 0.19, 6)
    cnt, _, _ = bale.triangle_agi(L)
    assert cnt == oracle.triangle_agi_mt(L.offset, L.nonzero)


def test_heavy_rows_with_malformed_neighbours(cuda, bale, mode):
    """A heavy row (>= 64 nonzeros, small label) whose neighbour row has bad
    offsets, and a heavy row that is not ascending: both are errors."""
    m = 100
    off, col = _clique(m)
    o = off.copy()
    o[70] = o[71] + 5  # row 69 ends after row 70 starts: offsets decrease at 70
    with pytest.raises(bale.BaleError):
        bale.triangle_agi(bale.SparseMatrix(o, col))
    c = col.copy()
    s = off[90]
    c[s + 10], c[s + 11] = c[s + 11], c[s + 10]  # row 90 (90 nonzeros) not ascending
    with pytest.raises(bale.BaleError):
        bale.triangle_agi(bale.SparseMatrix(off, c))
    assert bale.triangle_agi(bale.SparseMatrix(off, col))[0] == m * (m - 1) * (m - 2) // 6


def test_mixed_heavy_and_light_rows_match_oracle(cuda, bale, oracle, mode):
    """R-MAT with low edge factor plus a clique grafted on low labels: rows on
    both sides of the heavy threshold, heavy rows reading light rows."""
    L = bale.gen_rmat(15, 4, 0.57, 0.19, 0.19, 77)
    off, col = L.offset, L.nonzero
    m = 300  # make labels 0..299 a clique: rows 64..299 become heavy
    rows = []
    for i in range(L.numrows):
        r = col[off[i]:off[i + 1]]
        if i < m:
            r = np.union1d(r, np.arange(i, dtype=np.int64))
        rows.append(r)
    noff = np.zeros(L.numrows + 1, np.int64)
    noff[1:] = np.cumsum([r.size for r in rows])
    ncol = np.concatenate(rows).astype(np.int64)
    M = bale.SparseMatrix(noff, ncol)
    assert oracle.is_strict_lower_tidy(noff, ncol)
    assert bale.triangle_agi(M)[0] == oracle.triangle_agi(noff, ncol)[0]


def test_prepared_graph_counts_repeatedly(cuda, bale, oracle):
    """bale_triangle_prepare once, bale_triangle_count_prepared three times:
    three times the count, the probe tally each time, nothing flagged."""
    import torch

    L = bale.gen_rmat(14, 16, 0.57, 0.19, 0.19, 41)
    off = torch.from_numpy(L.offset).to(cuda)
    col = torch.from_numpy(L.nonzero).to(cuda)
    count = torch.zeros(1, dtype=torch.int64, device=cuda)
    work = torch.zeros(1, dtype=torch.int64, device=cuda)
    bad = torch.zeros(1, dtype=torch.int64, device=cuda)
    with bale.TrianglePrepared(off, col, bad=bad) as g:
        for _ in range(3):
            g.count(count, work)
    torch.cuda.synchronize()
    want = oracle.triangle_agi(L.offset, L.nonzero)[0]
    deg = np.diff(L.offset)
    rowid = np.repeat(np.arange(L.numrows), deg)
    pos = np.arange(L.nnz) - L.offset[rowid]
    assert int(count.item()) == 3 * want and int(bad.item()) == 0
    assert int(work.item()) == 3 * int(pos[deg[L.nonzero] > 0].sum())


def test_prepared_graph_malformed_is_flagged(cuda, bale):
    """A malformed matrix raises *bad at prepare time and counts nothing."""
    import torch

    off, col = _clique(70)
    c = col.copy()
    c[off[65] + 1], c[off[65] + 2] = c[off[65] + 2], c[off[65] + 1]
    d_off = torch.from_numpy(off).to(cuda)
    d_col = torch.from_numpy(c).to(cuda)
    count = torch.zeros(1, dtype=torch.int64, device=cuda)
    bad = torch.zeros(1, dtype=torch.int64, device=cuda)
    with bale.TrianglePrepared(d_off, d_col, bad=bad) as g:
        g.count(count)
    torch.cuda.synchronize()
    assert int(bad.item()) > 0 and int(count.item()) == 0


# The default mode picks the path per graph on the device (from 2^23
# nonzeros; below, the wedge path): wedges for graphs with hubs (R-MAT: pulls
# well above the pushes), the hybrid for graphs without (Erdos-Renyi) and for
# products of stars, whose thousands of wedges per nonzero make the wedge
# path far slower there.
# The count is exact either way; the work tally shows which path ran (it
# equals the forced mode's).
@pytest.mark.parametrize("graph,want", [("rmat20", 2), ("er20", 1), ("er64", 1), ("kron", 1), ("er16", 2)])
def test_default_mode_choice(cuda, bale, graph, want):
    if graph.startswith("rmat"):
        L = bale.gen_rmat(int(graph[4:]), 16, 0.57, 0.19, 0.19, 6)
    elif graph == "er20":
        L = bale.gen_erdos_renyi(1 << 20, 32.0 / (1 << 20), 7)
    elif graph == "er64":
        L = bale.gen_erdos_renyi(1 << 18, 128.0 / (1 << 18), 7)
    elif graph == "er16":  # below the size where the choice is made
        L = bale.gen_erdos_renyi(1 << 16, 32.0 / (1 << 16), 7)
    else:  # products of stars, large enough to be chosen for
        L = bale.gen_kronecker(1, [3, 4, 5, 9, 16, 25])
    cnt, sr, _ = bale.triangle_agi(L)
    bale.tune_set("tri.mode", want)
    try:
        fcnt, fsr, _ = bale.triangle_agi(L)
    finally:
        bale.tune_set("tri.mode", -1)
    assert cnt == fcnt and sr == fsr
    if graph == "kron":
        assert cnt == bale.kronecker_triangles(1, [3, 4, 5, 9, 16, 25])


def _transpose(oracle, off, col):
    uo, uc = oracle.transpose(off, col, off.size - 1)
    return uo, uc


@pytest.mark.parametrize("fn", DROPINS)
def test_alg1_with_u_transpose_counts_like_alg0(cuda, bale, oracle, golden, fn):
    """alg 1 (apps/triangle_src/triangle_agi.upc:100-136) with U = L^T, as the
    apps pass it (triangle.upc:306-307): every drop-in gives alg 0's count,
    on the reference's golden graphs and on R-MAT graphs."""
    d = golden("triangles")
    graphs = [(d[f"{g}/offset"], d[f"{g}/nonzero"], int(d[f"{g}/triangle_agi"][0])) for g in d["graphs"]]
    for scale in (10, 14):
        L = bale.gen_rmat(scale, 16, 0.57, 0.19, 0.19, 200 + scale)
        graphs.append((L.offset, L.nonzero, oracle.triangle_agi(L.offset, L.nonzero)[0]))
    for off, col, want in graphs:
        uo, uc = _transpose(oracle, off, col)
        L = bale.SparseMatrix(off, col)
        U = bale.SparseMatrix(uo, uc, off.size - 1)
        assert getattr(bale, fn)(L, U, 1)[0] == want


def test_alg1_with_other_upper_matrices_matches_oracle(cuda, bale, oracle):
    """alg 1 sums |U_i and U_j| over L's nonzeros for any tidy upper U: U from
    another graph, and L^T with a third of its entries dropped, against the
    oracle's restatement of the reference loop (pinned to the reference)."""
    rng = np.random.default_rng(11)
    for scale in (9, 12):
        L = bale.gen_rmat(scale, 16, 0.57, 0.19, 0.19, 300 + scale)
        L2 = bale.gen_rmat(scale, 8, 0.57, 0.19, 0.19, 400 + scale)
        keep = rng.random(L.nnz) < 0.67
        rows = np.repeat(np.arange(L.numrows), np.diff(L.offset))
        o3 = np.zeros(L.numrows + 1, np.int64)
        np.add.at(o3, rows[keep] + 1, 1)
        for moff, mcol in ((L2.offset, L2.nonzero), (np.cumsum(o3), np.ascontiguousarray(L.nonzero[keep]))):
            uo, uc = _transpose(oracle, moff, mcol)
            want = oracle.triangle_agi_alg1(L.offset, L.nonzero, uo, uc)[0]
            U = bale.SparseMatrix(uo, uc, L.numrows)
            for fn in ("triangle_agi", "triangle_exstack_push"):
                assert getattr(bale, fn)(L, U, 1)[0] == want


def test_alg1_needs_a_well_formed_u(cuda, bale, oracle):
    """alg 1 without U is an error (the reference returns -1 for a NULL U);
    so is a U that is not strictly upper, or not ascending; the library
    stays usable."""
    off, col = _clique(7)
    L = bale.SparseMatrix(off, col)
    with pytest.raises(bale.BaleError):
        bale.triangle_agi(L, None, 1)
    uo, uc = _transpose(oracle, off, col)
    bad = uc.copy()
    bad[0] = 0  # row 0 of U holding column 0: not strictly upper
    with pytest.raises(bale.BaleError):
        bale.triangle_agi(L, bale.SparseMatrix(uo, bad, 7), 1)
    bad = uc.copy()
    bad[0], bad[1] = bad[1], bad[0]  # not ascending
    with pytest.raises(bale.BaleError):
        bale.triangle_agi(L, bale.SparseMatrix(uo, bad, 7), 1)
    assert bale.triangle_agi(L, bale.SparseMatrix(uo, uc, 7), 1)[0] == 35


def test_alg1_full_size_rmat_scale22(cuda, bale, oracle):
    """alg 1 on the R-MAT scale-22 configuration with U = L^T: the count of
    alg 0, exact against the multi-threaded oracle."""
    L = bale.gen_rmat(22, 16, 0.57, 0.19, 0.19, 6)
    uo, uc = _transpose(oracle, L.offset, L.nonzero)
    cnt = bale.triangle_agi(L, bale.SparseMatrix(uo, uc, L.numrows), 1)[0]
    assert cnt == oracle.triangle_agi_mt(L.offset, L.nonzero)


def test_strategy_thresholds_steer_the_choice(cuda, bale):
    """The per-graph choice follows its tuned thresholds (the work-model rule
    tri.wedge_pull_pct / tri.wedge_push_per_nnz from tri.choose_min_nnz on):
    thresholds out of reach send an R-MAT graph to the hybrid, thresholds
    at zero to the wedges; the work tally shows which path ran and the count
    never changes."""
    L = bale.gen_rmat(14, 16, 0.57, 0.19, 0.19, 21)
    forced = {}
    for m in (1, 2):
        bale.tune_set("tri.mode", m)
        forced[m] = bale.triangle_agi(L)[:2]
    bale.tune_set("tri.mode", -1)
    try:
        bale.tune_set("tri.choose_min_nnz", 1)
        for pct, ppn, want in ((1 << 30, 1 << 40, 1), (0, 1 << 40, 2), (1 << 30, 0, 2)):
            bale.tune_set("tri.wedge_pull_pct", pct)
            bale.tune_set("tri.wedge_push_per_nnz", ppn)
            assert bale.triangle_agi(L)[:2] == forced[want], (pct, ppn)
    finally:
        for k in ("tri.choose_min_nnz", "tri.wedge_pull_pct", "tri.wedge_push_per_nnz"):
            bale.tune_set(k, -1)


@pytest.mark.parametrize("graph", ["rmat16", "rmat20", "kron_hubs", "erdos_renyi", "clique1800", "clique40"])
def test_dense_pairs_match_the_probes(cuda, bale, oracle, graph):
    """Wedge mode with the dense pairs (prefix longer than row j's bitmap
    words plus a margin) counted by bitmap AND instead of probes: off, at the
    default margin and at margin 0 (every eligible pair).  The count equals
    the oracle's and the work tally stays the probe count, sum of p over the
    nonzeros whose row j has columns."""
    import torch

    if graph.startswith("rmat"):
        L = bale.gen_rmat(int(graph[4:]), 16, 0.57, 0.19, 0.19, 11)
        off_h, col_h = L.offset, L.nonzero
    elif graph == "kron_hubs":
        L = bale.gen_kronecker(1, [1500, 3])
        off_h, col_h = L.offset, L.nonzero
    elif graph == "erdos_renyi":
        L = bale.gen_erdos_renyi(1 << 14, 64 / (1 << 14), 5)
        off_h, col_h = L.offset, L.nonzero
    else:
        off_h, col_h = _clique(int(graph[6:]))
    want = oracle.triangle_agi(off_h, col_h)[0]
    deg = np.diff(off_h)
    rowid = np.repeat(np.arange(off_h.size - 1), deg)
    pos = np.arange(col_h.size) - off_h[rowid]
    tally = int(pos[deg[col_h] > 0].sum())
    off = torch.from_numpy(off_h).to(cuda)
    col = torch.from_numpy(col_h).to(cuda)
    bale.tune_set("tri.mode", 2)
    try:
        for dense, ov in ((0, -1), (1, -1), (1, 0), (1, 7)):
            bale.tune_set("tri.dense", dense)
            bale.tune_set("tri.dense_ov", ov)
            count = torch.zeros(1, dtype=torch.int64, device=cuda)
            work = torch.zeros(1, dtype=torch.int64, device=cuda)
            bale.triangle_dev(off, col, count, work=work)
            torch.cuda.synchronize()
            assert int(count.item()) == want, (graph, dense, ov)
            assert int(work.item()) == tally, (graph, dense, ov)
    finally:
        for k in ("tri.mode", "tri.dense", "tri.dense_ov"):
            bale.tune_set(k, -1)
