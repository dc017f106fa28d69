"""Graph building on the device (bale_graph_build_dev, bale_gen_rmat_dev):
the same degree-ordered strictly lower CSR as the host builder, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lower_ref(u: np.ndarray, v: np.ndarray, n: int):
    """Restatement of the build on the CPU: the simple graph's strictly lower
    CSR with vertices relabelled by descending degree (ties by label)."""
    a, b = np.minimum(u, v), np.maximum(u, v)
    keep = a != b
    pairs = np.unique(np.stack([a[keep], b[keep]], 1), axis=0) if keep.any() else np.zeros((0, 2), np.int64)
    deg = np.bincount(pairs.ravel(), minlength=n)
    order = np.lexsort((np.arange(n), -deg))  # by descending degree, then label
    newid = np.empty(n, np.int64)
    newid[order] = np.arange(n)
    x, y = newid[pairs[:, 0]], newid[pairs[:, 1]]
    row, col = np.maximum(x, y), np.minimum(x, y)
    o = np.lexsort((col, row))
    row, col = row[o], col[o]
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, row + 1, 1)
    return np.cumsum(off), col


@pytest.mark.parametrize("scale", [4, 8, 11, 14, 17])
def test_rmat_on_device_equals_host(cuda, bale, scale):
    L = bale.gen_rmat(scale, 16, 0.57, 0.19, 0.19, 300 + scale)
    off, col = bale.gen_rmat_dev(scale, 16, 0.57, 0.19, 0.19, 300 + scale)
    np.testing.assert_array_equal(off.cpu().numpy(), L.offset)
    np.testing.assert_array_equal(col.cpu().numpy(), L.nonzero)


def test_rmat_other_parameters(cuda, bale):
    for (ef, a, b, c, seed) in ((4, 0.45, 0.15, 0.15, 9), (32, 0.25, 0.25, 0.25, 10), (1, 0.9, 0.05, 0.05, 11)):
        L = bale.gen_rmat(12, ef, a, b, c, seed)
        off, col = bale.gen_rmat_dev(12, ef, a, b, c, seed)
        np.testing.assert_array_equal(off.cpu().numpy(), L.offset)
        np.testing.assert_array_equal(col.cpu().numpy(), L.nonzero)


@pytest.mark.parametrize("n,m", [(1, 0), (1, 5), (2, 3), (37, 500), (1000, 20000), (70_001, 400_000)])
def test_edge_list_build_matches_restatement(cuda, bale, n, m):
    """Duplicates, both orientations and self loops in the input; any n."""
    import torch

    rng = np.random.default_rng(n + m)
    u = rng.integers(0, n, m).astype(np.int64)
    v = rng.integers(0, n, m).astype(np.int64)
    if m > 10:
        u[: m // 10], v[: m // 10] = v[m // 10: 2 * (m // 10)], u[m // 10: 2 * (m // 10)]  # reversed copies
        v[-5:] = u[-5:]  # self loops
    off, col = bale.graph_build_dev(torch.from_numpy(u).to(cuda), torch.from_numpy(v).to(cuda), n)
    want_off, want_col = _lower_ref(u, v, n)
    np.testing.assert_array_equal(off.cpu().numpy(), want_off)
    np.testing.assert_array_equal(col.cpu().numpy(), want_col)


def test_built_graph_counts_triangles_exactly(cuda, bale, oracle):
    """The device-built matrix is tidy and counts the same as the host one."""
    import torch

    off, col = bale.gen_rmat_dev(16, 16, 0.57, 0.19, 0.19, 5)
    assert oracle.is_strict_lower_tidy(off.cpu().numpy(), col.cpu().numpy())
    cnt = torch.zeros(1, dtype=torch.int64, device=cuda)
    bale.triangle_dev(off, col, cnt)
    torch.cuda.synchronize()
    L = bale.gen_rmat(16, 16, 0.57, 0.19, 0.19, 5)
    assert int(cnt.item()) == oracle.triangle_agi_mt(L.offset, L.nonzero)


def test_endpoint_outside_range_is_an_error(cuda, bale):
    import torch

    u = torch.tensor([0, 1, 2], dtype=torch.int64, device=cuda)
    v = torch.tensor([1, 5, -1], dtype=torch.int64, device=cuda)
    with pytest.raises(bale.BaleError, match="status 2|outside"):
        bale.graph_build_dev(u, v, 4)


def test_full_scale22_equals_host(cuda, bale):
    """The R-MAT scale-22 triangle input built on the device, identical."""
    L = bale.gen_rmat(22, 16, 0.57, 0.19, 0.19, 6)
    off, col = bale.gen_rmat_dev(22, 16, 0.57, 0.19, 0.19, 6)
    assert col.numel() == L.nnz
    assert np.array_equal(off.cpu().numpy(), L.offset)
    assert np.array_equal(col.cpu().numpy(), L.nonzero)
