"""Every graph on 1 to 5 vertices -- all 2^C(n,2) edge sets, 1,099 graphs --
counted on the GPU by each triangle path (merge, hybrid, wedge, the default)
and by the batched queue kernel, against a direct count of vertex triples.
Tiny exhaustive cases reach the corners random graphs miss: empty rows,
empty matrices, rows of one nonzero, every placement of a single wedge."""
from __future__ import annotations

import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _all_graphs(nmax: int = 5):
    """(offset, nonzero, triangles) of each strictly lower, ascending CSR on
    n = 1..nmax vertices, one per subset of the C(n,2) vertex pairs."""
    out = []
    for n in range(1, nmax + 1):
        pairs = [(i, j) for i in range(n) for j in range(i)]  # row-major, columns ascending
        for mask in range(1 << len(pairs)):
            rows = [[] for _ in range(n)]
            for b, (i, j) in enumerate(pairs):
                if mask >> b & 1:
                    rows[i].append(j)
            adj = {(i, j) for i, r in enumerate(rows) for j in r}
            want = sum(1 for a, b, c in itertools.combinations(range(n), 3)
                       if (b, a) in adj and (c, a) in adj and (c, b) in adj)
            off = np.zeros(n + 1, np.int64)
            off[1:] = np.cumsum([len(r) for r in rows])
            col = np.array([j for r in rows for j in r], np.int64)
            out.append((off, col, want))
    return out


GRAPHS = _all_graphs()


def test_graph_count_and_oracle(oracle):
    assert len(GRAPHS) == 1 + 2 + 8 + 64 + 1024
    assert all(oracle.triangle_agi(off, col)[0] == want for off, col, want in GRAPHS)
    # each of K_n's C(n,3) triangles lies in 1/8 of its 2^C(n,2) edge sets: 1 + 4*8 + 10*128
    assert sum(w for _, _, w in GRAPHS) == 1 + 32 + 1280


@pytest.mark.parametrize("tmode", [0, 1, 2, -1], ids=["merge", "hybrid", "wedge", "default"])
def test_every_tiny_graph_every_path(cuda, bale, tmode):
    bale.tune_set("tri.mode", tmode)
    try:
        wrong = []
        for k, (off, col, want) in enumerate(GRAPHS):
            cnt, _, _ = bale.triangle_agi(bale.SparseMatrix(off, col))
            if cnt != want:
                wrong.append((k, cnt, want))
        assert not wrong, wrong[:10]
    finally:
        bale.tune_set("tri.mode", -1)


def test_every_tiny_graph_in_one_batch(cuda, bale):
    import torch

    from bale_old_gb300 import batch

    offs = [torch.from_numpy(o).to(cuda) for o, _, _ in GRAPHS]
    cols = [torch.from_numpy(c).to(cuda) for _, c, _ in GRAPHS]
    counts = torch.zeros(len(GRAPHS), dtype=torch.int64, device=cuda)
    inst = [batch.triangles(o, c, counts[k:k + 1]) for k, (o, c) in enumerate(zip(offs, cols))]
    with batch.Batch(inst) as b:
        b.run()
        torch.cuda.synchronize()
        assert not b.bad().any()
        got = counts.cpu().numpy()
        b.run()  # replays add
        torch.cuda.synchronize()
        again = counts.cpu().numpy()
    want = np.array([w for _, _, w in GRAPHS], np.int64)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(again, 2 * want)
