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
