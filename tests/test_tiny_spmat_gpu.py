"""spmat's transpose and permutation on the GPU over every 0/1 matrix of a few
small shapes (3x3, 2x4, 4x2, 1x5, 5x1), with each row's columns in ascending
and in descending order, and permutations over every pair of row and column
permutations for a sample of them -- bit-exact against the oracle's one-PE
restatements of transpose_matrix_agi and permute_matrix_agi."""
from __future__ import annotations

import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(3, 3), (2, 4), (4, 2), (1, 5), (5, 1)]


def _matrices(r: int, c: int, descending: bool):
    for mask in range(1 << (r * c)):
        rows = [[j for j in range(c) if mask >> (i * c + j) & 1] for i in range(r)]
        if descending:
            rows = [row[::-1] for row in rows]
        off = np.zeros(r + 1, np.int64)
        off[1:] = np.cumsum([len(x) for x in rows])
        col = np.array([j for x in rows for j in x], np.int64)
        yield off, col


@pytest.mark.parametrize("descending", [False, True], ids=["ascending", "descending"])
@pytest.mark.parametrize("shape", SHAPES, ids=[f"{r}x{c}" for r, c in SHAPES])
def test_every_small_matrix_transposes_like_the_reference(cuda, bale, oracle, shape, descending):
    import torch

    r, c = shape
    wrong = []
    for k, (off, col) in enumerate(_matrices(r, c, descending)):
        toff, tcol = bale.transpose_dev(torch.from_numpy(off).to(cuda), torch.from_numpy(col).to(cuda), c)
        woff, wcol = oracle.transpose(off, col, c)
        if not (np.array_equal(toff.cpu().numpy(), woff) and np.array_equal(tcol.cpu().numpy(), wcol)):
            wrong.append(k)
    assert not wrong, wrong[:10]


@pytest.mark.parametrize("shape", [(3, 3), (2, 4), (4, 2)], ids=["3x3", "2x4", "4x2"])
def test_small_matrices_permute_like_the_reference_under_every_permutation(cuda, bale, oracle, shape):
    import torch

    r, c = shape
    mats = list(_matrices(r, c, descending=False))[::37]  # a spread of the 2^(rc) patterns
    mats += list(_matrices(r, c, descending=True))[-1:]    # the full matrix, rows descending
    wrong = []
    for rp in itertools.permutations(range(r)):
        rinv = np.array(rp, np.int64)
        for cp in itertools.permutations(range(c)):
            cinv = np.array(cp, np.int64)
            drinv, dcinv = torch.from_numpy(rinv).to(cuda), torch.from_numpy(cinv).to(cuda)
            for k, (off, col) in enumerate(mats):
                poff, pcol = bale.permute_dev(torch.from_numpy(off).to(cuda), torch.from_numpy(col).to(cuda),
                                              c, drinv, dcinv)
                woff, wcol = oracle.permute(off, col, rinv, cinv)
                if not (np.array_equal(poff.cpu().numpy(), woff) and np.array_equal(pcol.cpu().numpy(), wcol)):
                    wrong.append((rp, cp, k))
    assert not wrong, wrong[:10]
