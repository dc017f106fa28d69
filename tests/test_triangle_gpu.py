"""Triangle counting on the GPU, through the C ABI: exact int64 counts equal
to the reference's (golden vectors, Kronecker closed forms) and to the
oracle on seeded R-MAT and Erdos-Renyi graphs up to the full scale-22 size."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DROPINS = ("triangle_agi", "triangle_exstack_push", "triangle_exstack2_push",
           "triangle_convey_push", "triangle_agi_iter")


def test_golden_graphs_all_dropins(cuda, bale, golden):
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


@pytest.mark.parametrize("mode,specs", [(1, [3, 4, 5, 9]), (2, [3, 4, 5, 9, 2]), (0, [5, 9, 4]),
                                        (1, [1, 4, 9, 16, 25]), (1, [2000, 2]), (2, [1500, 3])])
def test_kronecker_closed_forms_including_hub_rows(cuda, bale, mode, specs):
    """Star products have hub rows far longer than a warp's shared-memory slot."""
    L = bale.gen_kronecker(mode, specs)
    cnt, _, _ = bale.triangle_agi(L)
    assert cnt == bale.kronecker_triangles(mode, specs)


@pytest.mark.parametrize("scale", [6, 10, 14, 16])
def test_rmat_matches_oracle(cuda, bale, oracle, scale):
    L = bale.gen_rmat(scale, 16, 0.57, 0.19, 0.19, 100 + scale)
    cnt, sr, _ = bale.triangle_agi(L)
    assert cnt == oracle.triangle_agi_mt(L.offset, L.nonzero)
    # the device tally is the number of row-j elements scanned: the pulls of
    # every (i,j) except the first nonzero of each row
    deg = np.diff(L.offset)
    nf = np.ones(L.nnz, bool)
    nf[L.offset[:-1][deg > 0]] = False
    assert sr == int(deg[L.nonzero[nf]].sum())


def test_erdos_renyi_matches_oracle(cuda, bale, oracle):
    n = 1 << 16
    L = bale.gen_erdos_renyi(n, 32.0 / n, 7)
    assert bale.triangle_agi(L)[0] == oracle.triangle_agi_mt(L.offset, L.nonzero)


def _clique(m: int):
    off = np.zeros(m + 1, np.int64)
    off[1:] = np.cumsum(np.arange(m))
    col = np.concatenate([np.arange(i, dtype=np.int64) for i in range(m)]) if m > 1 else np.zeros(0, np.int64)
    return off, col


@pytest.mark.parametrize("m", [0, 1, 2, 3, 40, 1025, 1800])
def test_cliques_long_rows_and_tiny_graphs(cuda, bale, m):
    off, col = _clique(m)
    L = bale.SparseMatrix(off, col)
    assert bale.triangle_agi(L)[0] == m * (m - 1) * (m - 2) // 6


def test_malformed_matrices_are_errors_not_faults(cuda, bale):
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


def test_full_size_rmat_scale22(cuda, bale, oracle):
    """The R-MAT scale-22 configuration, exact against the multi-threaded oracle."""
    L = bale.gen_rmat(22, 16, 0.57, 0.19, 0.19, 6)
    cnt, _, _ = bale.triangle_agi(L)
    assert cnt == oracle.triangle_agi_mt(L.offset, L.nonzero)
