"""The radix sort under the graph build, transpose_matrix, the MatrixMarket
reader and randperm: the single-sweep passes (tile look-back) against the
three-step passes (histogram, scan, scatter), and the bounded look-back wait
giving up with BALE_ETIMEDOUT while the output stays exact."""
from __future__ import annotations

import contextlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BALE_ETIMEDOUT = 5


@contextlib.contextmanager
def knob(bale, name, value):
    bale.tune_set(name, value)
    try:
        yield
    finally:
        bale.tune_set(name, -1)


def _np(t):
    return t.cpu().numpy()


@pytest.mark.parametrize("scale", [1, 6, 12, 18, 21])
def test_single_sweep_build_equals_three_step(cuda, bale, scale):
    """R-MAT graphs from 2 to 2^21 vertices (a part tile, one tile, thousands)."""
    a = bale.gen_rmat_dev(scale, 16, 0.57, 0.19, 0.19, scale, device=cuda)
    with knob(bale, "sort.onesweep", 0):
        b = bale.gen_rmat_dev(scale, 16, 0.57, 0.19, 0.19, scale, device=cuda)
    np.testing.assert_array_equal(_np(a[0]), _np(b[0]))
    np.testing.assert_array_equal(_np(a[1]), _np(b[1]))


@pytest.mark.parametrize("scale", [9, 20])
def test_single_sweep_transpose_equals_three_step(cuda, bale, oracle, scale):
    off, col = bale.gen_rmat_dev(scale, 16, 0.57, 0.19, 0.19, 3, device=cuda)
    n = off.numel() - 1
    to, tc = bale.transpose_dev(off, col, n)
    with knob(bale, "sort.onesweep", 0):
        uo, uc = bale.transpose_dev(off, col, n)
    np.testing.assert_array_equal(_np(to), _np(uo))
    np.testing.assert_array_equal(_np(tc), _np(uc))
    wo, wc = oracle.transpose(_np(off), _np(col), n)
    np.testing.assert_array_equal(_np(to), wo)
    np.testing.assert_array_equal(_np(tc), wc)


def test_single_sweep_region_pass_of_randperm(cuda, bale):
    """rand_permp groups its throws by slot region with one radix pass above
    2^21 elements; both pass forms give the same permutation."""
    n = (1 << 23) + 12345
    a = bale.rand_perm_dev(n, 77, device=cuda)
    with knob(bale, "sort.onesweep", 0):
        b = bale.rand_perm_dev(n, 77, device=cuda)
    np.testing.assert_array_equal(_np(a), _np(b))
    assert np.array_equal(np.sort(_np(a)), np.arange(n))


def test_lookback_wait_gives_up_with_status(cuda, bale, oracle):
    """Tile 0 of every pass withholds its counts (a test knob), so its
    successors' bounded waits run out: the call returns BALE_ETIMEDOUT, and
    the blocks' recount from the earlier tiles' keys keeps the transpose
    exact.  Without the knob the same call succeeds."""
    import torch

    off, col = bale.gen_rmat_dev(16, 16, 0.57, 0.19, 0.19, 5, device=cuda)
    n, nnz = off.numel() - 1, col.numel()
    wo, wc = oracle.transpose(_np(off), _np(col), n)
    toff = torch.full((n + 1,), -1, dtype=torch.int64, device=cuda)
    tcol = torch.full((nnz,), -1, dtype=torch.int64, device=cuda)
    with knob(bale, "sort.test_withhold", 1), knob(bale, "sort.lookback_spins", 64):
        rc = bale._lib.bale_transpose_dev(off.data_ptr(), col.data_ptr(), n, n, nnz, toff.data_ptr(),
                                          tcol.data_ptr(), None)
        torch.cuda.synchronize()
        assert rc == BALE_ETIMEDOUT
        assert "gave up" in bale._last_error()
        np.testing.assert_array_equal(_np(toff), wo)
        np.testing.assert_array_equal(_np(tcol), wc)
        with pytest.raises(bale.BaleError, match="status 5"):
            bale.gen_rmat_dev(12, 16, 0.57, 0.19, 0.19, 5, device=cuda)
    to, tc = bale.transpose_dev(off, col, n)
    np.testing.assert_array_equal(_np(to), wo)
    np.testing.assert_array_equal(_np(tc), wc)
