"""MatrixMarket files (host side): the writer produces the reference's bytes,
the header reader takes what the reference's reader takes."""
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
