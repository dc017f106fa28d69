"""MatrixMarket files and binary datasets (host side): the writers produce
the reference's bytes, the header readers take what the reference's readers
take."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("tag", ["rmat8_lower", "rect_300x517"])
def test_writer_matches_reference_bytes(bale, golden, tmp_path, tag):
    d = golden("spmat")
    L = bale.SparseMatrix(d[f"{tag}/offset"], d[f"{tag}/nonzero"], int(d[f"{tag}/numcols"][0]))
    out = tmp_path / f"{tag}.mm"
    bale.write_matrix_mm(L, out)
    assert out.read_bytes() == (GOLDEN / f"{tag}.mm").read_bytes()


def test_header_reader(bale, tmp_path):
    assert bale.mm_header(GOLDEN / "rmat8_lower.mm")[:3] == (256, 256, 2144)
    assert bale.mm_header(GOLDEN / "unordered_integer.mm") == (5, 7, 9, 3)
    p = tmp_path / "c.mm"
    p.write_text("%%MatrixMarket matrix coordinate pattern\n% a comment\n%another\n3 4 2\n1 1\n3 4\n")
    assert bale.mm_header(p) == (3, 4, 2, 2)
    for bad in ("%%MatrixMarket matrix array real\n2 2\n", "%%MatrixMarket vector coordinate pattern\n1 1 1\n",
                "MatrixMarket matrix coordinate pattern\n1 1 1\n", "%%MatrixMarket matrix coordinate real\n1 1 1\n",
                "%%MatrixMarket matrix coordinate pattern\n2 x 1\n"):
        p.write_text(bad)
        with pytest.raises(bale.BaleError):
            bale.mm_header(p)
    with pytest.raises(bale.BaleError):
        bale.mm_header(tmp_path / "missing.mm")


DS_FILES = ("metadata", "rowcnt_0", "nonzero_0")


@pytest.mark.parametrize("tag", ["rmat8_lower", "rect_300x517"])
def test_dataset_writer_matches_reference_bytes(bale, golden, tmp_path, tag):
    d = golden("spmat")
    L = bale.SparseMatrix(d[f"{tag}/offset"], d[f"{tag}/nonzero"], int(d[f"{tag}/numcols"][0]))
    out = tmp_path / f"ds_{tag}"
    bale.write_sparse_matrix(L, out)
    assert sorted(p.name for p in out.iterdir()) == sorted(DS_FILES)
    for f in DS_FILES:
        assert (out / f).read_bytes() == (GOLDEN / f"ds_{tag}" / f).read_bytes(), f


@pytest.mark.parametrize("tag", ["rmat8_lower", "rect_300x517"])
def test_dataset_oracle_matches_reference_bytes(oracle, golden, tmp_path, tag):
    d = golden("spmat")
    out = tmp_path / f"ds_{tag}"
    oracle.write_dataset(d[f"{tag}/offset"], d[f"{tag}/nonzero"], int(d[f"{tag}/numcols"][0]), out)
    for f in DS_FILES:
        assert (out / f).read_bytes() == (GOLDEN / f"ds_{tag}" / f).read_bytes(), f


def test_dataset_header_reader(bale, tmp_path):
    assert bale.sparse_matrix_header(GOLDEN / "ds_rmat8_lower") == (256, 256, 2144, 1)
    assert bale.sparse_matrix_header(GOLDEN / "ds_rect_300x517")[3] == 1
    (tmp_path / "metadata").write_text("7\n9\n11\n3\n")
    assert bale.sparse_matrix_header(tmp_path) == (7, 9, 11, 3)
    for bad in ("7\n9\n11\n", "7\n9\n11\n0\n", "-1\n9\n11\n1\n", "x\n"):
        (tmp_path / "metadata").write_text(bad)
        with pytest.raises(bale.BaleError):
            bale.sparse_matrix_header(tmp_path)
    with pytest.raises(bale.BaleError):
        bale.sparse_matrix_header(tmp_path / "missing")


def _small_matrices(r: int, c: int, descending: bool):
    for mask in range(1 << (r * c)):
        rows = [[j for j in range(c) if mask >> (i * c + j) & 1] for i in range(r)]
        if descending:
            rows = [row[::-1] for row in rows]
        off = np.zeros(r + 1, np.int64)
        off[1:] = np.cumsum([len(x) for x in rows])
        yield off, np.array([j for x in rows for j in x], np.int64)


def test_writers_match_reference_bytes_on_every_small_matrix(bale, tmp_path, monkeypatch):
    """The library's host writers against the reference's own, byte for byte,
    on every 0/1 matrix of five small shapes with rows in either order; the
    header readers give back the sizes."""
    from oracle.pyoracle import REF_LIB, Reference

    if not REF_LIB.exists():
        pytest.skip("oracle/_ref is built only where the reference tree exists")
    ref = Reference()
    monkeypatch.chdir(tmp_path)  # short relative names: the reference's file names are 64-byte buffers
    import shutil

    for r, c in [(3, 3), (2, 4), (4, 2), (1, 5), (5, 1)]:
        for desc in (False, True):
            for off, col in _small_matrices(r, c, desc):
                L = bale.SparseMatrix(off, col, numcols=c)
                bale.write_matrix_mm(L, "ours.mm")
                ref.write_mm(off, col, c, "ref.mm")
                assert Path("ours.mm").read_bytes() == Path("ref.mm").read_bytes(), (r, c, off, col)
                assert bale.mm_header("ours.mm") == (r, c, col.size, 2)
                bale.write_sparse_matrix(L, "o")
                ref.write_dataset(off, col, c, "r")
                for name in ("metadata", "rowcnt_0", "nonzero_0"):
                    assert Path("o", name).read_bytes() == Path("r", name).read_bytes(), (r, c, name)
                assert bale.sparse_matrix_header("o") == (r, c, col.size, 1)
                shutil.rmtree("o")
                shutil.rmtree("r")
