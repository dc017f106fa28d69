"""Host side of the serving loop: request constructors, argument checks and
the Poisson arrival trace.  No server is created (that needs a GPU)."""
from __future__ import annotations

import numpy as np
import pytest

from bale_old_gb300 import serve


def test_request_constructors_carry_kind_and_arrays():
    idx = np.arange(10, dtype=np.int64)
    out = np.zeros(10, np.int64)
    r = serve.ig(3, idx, out, arrival=0.5, shift=16)
    assert (r.kind, r.obj, r.arrival, r.shift) == (serve.IG, 3, 0.5, 16)
    assert r.index is idx and r.out is out
    h = serve.histo(1, idx, arrival=0.25)
    assert (h.kind, h.obj, h.out) == (serve.HISTO, 1, None)
    one = np.zeros(1, np.int64)
    t = serve.triangles(2, one)
    assert (t.kind, t.index, t.out) == (serve.TRIANGLES, None, one)


def test_request_constructors_refuse_short_outputs():
    with pytest.raises(ValueError):
        serve.ig(0, np.zeros(5, np.int64), np.zeros(4, np.int64))
    with pytest.raises(ValueError):
        serve.triangles(0, np.zeros(0, np.int64))


@pytest.mark.parametrize("bad", [np.zeros(4, np.int32), np.zeros((4, 2), np.int64)[:, 0], [1, 2, 3]])
def test_array_check_wants_contiguous_int64(bad):
    with pytest.raises(TypeError):
        serve._check(bad, "index")
    serve._check(None, "out")
    serve._check(np.zeros(4, np.int64), "index")


def test_poisson_arrivals():
    a = serve.poisson_arrivals(20000, 1000.0, 7)
    assert a.shape == (20000,) and np.all(np.diff(a) > 0) and a[0] > 0
    gaps = np.diff(np.concatenate([[0.0], a]))
    assert abs(gaps.mean() - 1e-3) < 5e-5          # mean gap 1/rate
    assert abs(gaps.std() / gaps.mean() - 1) < 0.05  # exponential: cv = 1
    assert np.array_equal(a, serve.poisson_arrivals(20000, 1000.0, 7))
    assert np.array_equal(serve.poisson_arrivals(5, 0.0, 1), np.zeros(5))  # rate 0: all at once
