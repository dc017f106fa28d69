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


def _dev(a, cuda):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def test_transpose_and_permute_match_reference_golden(cuda, bale, golden):
    d = golden("spmat")
    for t in d["mats"]:
        off, col, nc = d[f"{t}/offset"], d[f"{t}/nonzero"], int(d[f"{t}/numcols"][0])
        to, tc = bale.transpose_dev(_dev(off, cuda), _dev(col, cuda), nc)
        np.testing.assert_array_equal(to.cpu().numpy(), d[f"{t}/t_offset"], err_msg=str(t))
        np.testing.assert_array_equal(tc.cpu().numpy(), d[f"{t}/t_nonzero"], err_msg=str(t))
        po, pc = bale.permute_dev(_dev(off, cuda), _dev(col, cuda), nc, _dev(d[f"{t}/rperminv"], cuda),
                                  _dev(d[f"{t}/cperminv"], cuda))
        np.testing.assert_array_equal(po.cpu().numpy(), d[f"{t}/p_offset"], err_msg=str(t))
        np.testing.assert_array_equal(pc.cpu().numpy(), d[f"{t}/p_nonzero"], err_msg=str(t))


def test_rand_perm_matches_reference_golden(cuda, bale, golden):
    d = golden("spmat")
    for p in d["perms"]:
        _, n, seed = str(p).split("_")
        np.testing.assert_array_equal(bale.rand_perm_dev(int(n), int(seed)).cpu().numpy(), d[p], err_msg=str(p))


@pytest.mark.parametrize("n,seed", [(3, 5), (4097, 77), (1 << 20, 2024), (3_000_001, 9)])
def test_rand_perm_matches_oracle_at_size(cuda, bale, oracle, n, seed):
    np.testing.assert_array_equal(bale.rand_perm_dev(n, seed).cpu().numpy(), oracle.rand_perm(n, seed))


def test_rand_perm_exstack_matches_reference_golden(cuda, bale, golden):
    d = golden("spmat")
    for p in d["xperms"]:
        _, n, seed, b = str(p).split("_")
        got = bale.rand_perm_exstack_dev(int(n), int(seed), int(b)).cpu().numpy()
        np.testing.assert_array_equal(got, d[p], err_msg=str(p))
    np.testing.assert_array_equal(bale.rand_perm_exstack_dev(100_000, 31).cpu().numpy(), d["permp_100000_31"])


# buffers far below n (most rounds full), of one dart, near n, and above n
@pytest.mark.parametrize("n,seed,b", [(4097, 77, 1024), (1 << 20, 2024, 1024), (3_000_001, 9, 1024),
                                      (200_000, 4, 1), (300_000, 6, 299_999), (50_000, 12, 1 << 40),
                                      (1 << 20, 5, 65_536)])
def test_rand_perm_exstack_matches_oracle_at_size(cuda, bale, oracle, n, seed, b):
    got = bale.rand_perm_exstack_dev(n, seed, b).cpu().numpy()
    np.testing.assert_array_equal(got, oracle.rand_perm_exstack(n, seed, b))


def test_rand_perm_exstack2_matches_reference_golden(cuda, bale, golden):
    """rand_permp_exstack2 (spmat/spmat_exstack2.upc:60-73) as the reference
    computes it, against its own outputs, and equal to the exstack form."""
    d = golden("spmat")
    for p in d["x2perms"]:
        _, n, seed, b = str(p).split("_")
        got = bale.rand_perm_exstack2_dev(int(n), int(seed), int(b)).cpu().numpy()
        np.testing.assert_array_equal(got, d[p], err_msg=str(p))
    np.testing.assert_array_equal(bale.rand_perm_exstack2_dev(3000, 2, 4096).cpu().numpy(),
                                  bale.rand_perm_exstack_dev(3000, 2, 4096).cpu().numpy())


def _libc():
    import ctypes

    libc = ctypes.CDLL(None)
    libc.srand48.argtypes = [ctypes.c_long]
    libc.srand48.restype = None
    libc.lrand48.restype = ctypes.c_long
    return libc


def test_rand_perm_seed_zero_continues_the_c_library_stream(cuda, bale, oracle):
    """Seed 0 continues the C library's drand48 stream and every call leaves
    it just past the reference's last draw: sequences of seeded and seed-0
    calls on the device give the oracle's permutations (pinned to the
    reference on the same sequences) and leave the same stream behind, read
    out with a final lrand48()."""
    libc = _libc()

    def run(impl, c):
        if c[0] == "agi":
            out = impl.rand_perm_dev(c[1], c[2]) if impl is bale else impl.rand_perm(c[1], c[2])
        else:
            out = (impl.rand_perm_exstack_dev(c[1], c[2], c[3]) if impl is bale
                   else impl.rand_perm_exstack(c[1], c[2], c[3]))
        return out.cpu().numpy() if impl is bale else out

    sequences = [
        [("agi", 10, 0), ("agi", 1, 0), ("x", 7, 0, 3), ("x", 100, 0, 1024), ("x", 33, 0, 1)],
        [("agi", 5, 9), ("agi", 12, 0), ("x", 40, 4, 2), ("x", 40, 0, 2), ("agi", 3, 0)],
        [("x", 1000, 0, 7), ("agi", 1000, 0), ("x", 64, 0, 64), ("x", 65, 0, 64)],
        [("agi", 100_000, 0), ("x", 70_001, 0, 1024), ("agi", 4097, 77), ("x", 5000, 0, 64)],
    ]
    for start in (0, 5, 123456):
        for calls in sequences:
            libc.srand48(start)
            dev = [run(bale, c) for c in calls]
            dev_next = libc.lrand48()
            libc.srand48(start)
            orc = [run(oracle, c) for c in calls]
            orc_next = libc.lrand48()
            for c, a, b in zip(calls, dev, orc):
                np.testing.assert_array_equal(a, b, err_msg=f"start {start} {c}")
            assert dev_next == orc_next, (start, calls)


def test_rand_perm_exstack_rejects_bad_arguments(cuda, bale):
    with pytest.raises(bale.BaleError):
        bale.rand_perm_exstack_dev(100, 1, 0)
    with pytest.raises(bale.BaleError):
        bale.rand_perm_exstack_dev(-1, 1, 1024)
    assert bale.rand_perm_exstack_dev(0, 1, 1024).numel() == 0


@pytest.mark.parametrize("scale", [12, 18])
def test_transpose_and_permute_match_oracle_at_size(cuda, bale, oracle, scale):
    L = bale.gen_rmat(scale, 16, 0.57, 0.19, 0.19, scale)
    n = L.numrows
    to, tc = bale.transpose_dev(_dev(L.offset, cuda), _dev(L.nonzero, cuda), n)
    wo, wc = oracle.transpose(L.offset, L.nonzero, n)
    np.testing.assert_array_equal(to.cpu().numpy(), wo)
    np.testing.assert_array_equal(tc.cpu().numpy(), wc)
    rinv = oracle.rand_perm(n, 11)
    cinv = oracle.rand_perm(n, 12)
    po, pc = bale.permute_dev(_dev(L.offset, cuda), _dev(L.nonzero, cuda), n, _dev(rinv, cuda), _dev(cinv, cuda))
    qo, qc = oracle.permute(L.offset, L.nonzero, rinv, cinv)
    np.testing.assert_array_equal(po.cpu().numpy(), qo)
    np.testing.assert_array_equal(pc.cpu().numpy(), qc)


def test_spmat_ops_reject_bad_input(cuda, bale):
    off = np.array([0, 2, 3], np.int64)
    col = np.array([0, 5, 1], np.int64)  # column 5 outside a 3-column matrix
    with pytest.raises(bale.BaleError, match="status 2"):
        bale.transpose_dev(_dev(off, cuda), _dev(col, cuda), 3)
    col[1] = 2
    with pytest.raises(bale.BaleError, match="status 2"):  # not a permutation
        bale.permute_dev(_dev(off, cuda), _dev(col, cuda), 3, _dev(np.array([0, 0], np.int64), cuda),
                         _dev(np.array([2, 1, 0], np.int64), cuda))
    po, pc = bale.permute_dev(_dev(off, cuda), _dev(col, cuda), 3, _dev(np.array([1, 0], np.int64), cuda),
                              _dev(np.array([2, 1, 0], np.int64), cuda))
    np.testing.assert_array_equal(po.cpu().numpy(), [0, 1, 3])
    np.testing.assert_array_equal(pc.cpu().numpy(), [1, 2, 0])


def test_matrix_market_read_matches_reference_golden(cuda, bale, golden):
    from pathlib import Path

    gdir = Path(__file__).resolve().parent / "golden"
    d = golden("spmat")
    for f in d["mm_files"]:
        off, col, nc = bale.read_matrix_mm_dev(gdir / str(f))
        np.testing.assert_array_equal(off.cpu().numpy(), d[f"mm/{f}/offset"], err_msg=str(f))
        np.testing.assert_array_equal(col.cpu().numpy(), d[f"mm/{f}/nonzero"], err_msg=str(f))
        assert nc == int(d[f"mm/{f}/numcols"][0])


def test_matrix_market_round_trip_at_size(cuda, bale, tmp_path):
    L = bale.gen_rmat(17, 16, 0.57, 0.19, 0.19, 23)
    p = tmp_path / "rmat17.mm"
    bale.write_matrix_mm(L, p)
    off, col, nc = bale.read_matrix_mm_dev(p)
    assert nc == L.numcols
    np.testing.assert_array_equal(off.cpu().numpy(), L.offset)
    np.testing.assert_array_equal(col.cpu().numpy(), L.nonzero)


def test_matrix_market_tolerates_blanks_crlf_and_comments(cuda, bale, tmp_path):
    p = tmp_path / "loose.mm"
    p.write_bytes(b"%%MatrixMarket matrix coordinate pattern\r\n% made by hand\r\n3 3 4\r\n"
                  b"  2 1\r\n\r\n3\t1 \r\n% a comment between entries\n3 2\n1 3")
    off, col, nc = bale.read_matrix_mm_dev(p)
    np.testing.assert_array_equal(off.cpu().numpy(), [0, 1, 2, 4])
    np.testing.assert_array_equal(col.cpu().numpy(), [2, 0, 0, 1])


@pytest.mark.parametrize("body", ["3 3 2\n1 1\n", "3 3 2\n1 1\n2 2\n3 3\n", "3 3 2\n1 1\n4 1\n",
                                  "3 3 2\n1 1\n2 0\n", "3 3 2\n1 1\n2 x\n", "3 3 2\n1 1\n2 2 2\n"])
def test_matrix_market_malformed_is_an_error(cuda, bale, tmp_path, body):
    p = tmp_path / "bad.mm"
    p.write_text("%%MatrixMarket matrix coordinate pattern\n" + body)
    with pytest.raises(bale.BaleError):
        bale.read_matrix_mm_dev(p)


# ---------------------------------------------------------------- binary datasets
DS_FILES = ("metadata", "rowcnt_0", "nonzero_0")


def _golden_dir():
    from pathlib import Path

    return Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("tag", ["rmat8_lower", "rect_300x517"])
def test_dataset_device_writer_matches_reference_bytes(cuda, bale, golden, tmp_path, tag):
    d = golden("spmat")
    off, col, nc = d[f"{tag}/offset"], d[f"{tag}/nonzero"], int(d[f"{tag}/numcols"][0])
    bale.write_sparse_matrix_dev(tmp_path / "ds", _dev(off, cuda), _dev(col, cuda), nc)
    for f in DS_FILES:
        assert (tmp_path / "ds" / f).read_bytes() == (_golden_dir() / f"ds_{tag}" / f).read_bytes(), f


@pytest.mark.parametrize("tag", ["rmat8_lower", "rect_300x517"])
def test_dataset_reader_reads_reference_files(cuda, bale, golden, tag):
    d = golden("spmat")
    off, col, nc = bale.read_sparse_matrix_dev(_golden_dir() / f"ds_{tag}")
    assert nc == int(d[f"{tag}/numcols"][0])
    np.testing.assert_array_equal(off.cpu().numpy(), d[f"{tag}/offset"])
    np.testing.assert_array_equal(col.cpu().numpy(), d[f"{tag}/nonzero"])


@pytest.mark.parametrize("writers", [2, 3, 7, 301, 1000])
def test_dataset_writer_blocks(cuda, bale, golden, tmp_path, writers):
    """W writers: the w-th block of (n + W - w - 1) / W rows; the files put
    together are the one-writer files."""
    d = golden("spmat")
    tag = "rect_300x517"
    off, col, nc = d[f"{tag}/offset"], d[f"{tag}/nonzero"], int(d[f"{tag}/numcols"][0])
    n = off.size - 1
    out = tmp_path / "ds"
    bale.write_sparse_matrix_dev(out, _dev(off, cuda), _dev(col, cuda), nc, nwriters=writers)
    assert (out / "metadata").read_text().split() == [str(n), str(nc), str(col.size), str(writers)]
    rc = [np.fromfile(out / f"rowcnt_{w}", np.int64) for w in range(writers)]
    assert [r.size for r in rc] == [(n + writers - w - 1) // writers for w in range(writers)]
    g = _golden_dir() / f"ds_{tag}"
    assert b"".join(r.tobytes() for r in rc) == (g / "rowcnt_0").read_bytes()
    assert b"".join((out / f"nonzero_{w}").read_bytes() for w in range(writers)) == (g / "nonzero_0").read_bytes()
    r_off, r_col, r_nc = bale.read_sparse_matrix_dev(out)
    assert r_nc == nc
    np.testing.assert_array_equal(r_off.cpu().numpy(), off)
    np.testing.assert_array_equal(r_col.cpu().numpy(), col)


def test_dataset_round_trip_at_size(cuda, bale, tmp_path):
    off, col = bale.gen_rmat_dev(18, 16, 0.57, 0.19, 0.19, 29)
    n = off.numel() - 1
    for writers in (1, 5):
        out = tmp_path / f"ds{writers}"
        bale.write_sparse_matrix_dev(out, off, col, n, nwriters=writers)
        r_off, r_col, nc = bale.read_sparse_matrix_dev(out)
        assert nc == n
        assert torch_equal(r_off, off) and torch_equal(r_col, col)


def torch_equal(a, b) -> bool:
    import torch

    return a.shape == b.shape and bool(torch.equal(a, b))


def test_dataset_empty_and_tiny(cuda, bale, tmp_path):
    off = np.zeros(4, np.int64)
    bale.write_sparse_matrix_dev(tmp_path / "e", _dev(off, cuda), _dev(np.zeros(1, np.int64), cuda)[:0], 3,
                                 nwriters=5)
    r_off, r_col, nc = bale.read_sparse_matrix_dev(tmp_path / "e")
    assert nc == 3 and r_col.numel() == 0
    np.testing.assert_array_equal(r_off.cpu().numpy(), off)


def _write_ds(tmp_path, meta, rowcnts, nonzeros):
    out = tmp_path / "bad"
    out.mkdir(exist_ok=True)
    (out / "metadata").write_text("".join(f"{v}\n" for v in meta))
    for w, (r, z) in enumerate(zip(rowcnts, nonzeros)):
        np.asarray(r, np.int64).tofile(out / f"rowcnt_{w}")
        np.asarray(z, np.int64).tofile(out / f"nonzero_{w}")
    return out


@pytest.mark.parametrize("case", [
    ((3, 4, 3, 1), [[1, 1, 1]], [[0, 1]]),                # one column short
    ((3, 4, 3, 1), [[1, 1]], [[0, 1, 2]]),                # one row length short
    ((3, 4, 3, 1), [[1, -1, 3]], [[0, 1, 2]]),            # a negative length
    ((3, 4, 3, 1), [[1, 1, 1]], [[0, 4, 2]]),             # a column past numcols
    ((3, 4, 3, 1), [[1, 1, 1]], [[0, -1, 2]]),            # a negative column
    ((4, 4, 4, 2), [[2, 1], [0, 1]], [[0, 1], [2, 3]]),   # lengths of writer 0 run into writer 1's columns
    ((3, 4, 3, 2), [[1, 1, 1], []], [[0, 1, 2], []]),     # writer blocks of the wrong sizes
])
def test_dataset_malformed_is_an_error(cuda, bale, tmp_path, case):
    out = _write_ds(tmp_path, *case)
    with pytest.raises(bale.BaleError):
        bale.read_sparse_matrix_dev(out)


def test_dataset_missing_file_and_bad_csr(cuda, bale, tmp_path):
    out = _write_ds(tmp_path, (2, 2, 1, 2), [[1], [0]], [[0], []])
    (out / "nonzero_1").unlink()
    with pytest.raises(bale.BaleError):
        bale.read_sparse_matrix_dev(out)
    with pytest.raises(bale.BaleError):
        bale.write_sparse_matrix_dev(tmp_path / "w", _dev(np.array([0, 2, 1], np.int64), cuda),
                                     _dev(np.array([0, 1], np.int64), cuda), 2)
    with pytest.raises(bale.BaleError):
        bale.write_sparse_matrix_dev(tmp_path / "w", _dev(np.array([0, 1, 2], np.int64), cuda),
                                     _dev(np.array([0, 2], np.int64), cuda), 2)
