"""The serving loop (bale_server_* in include/bale_gb300.h): resident tables,
counters and graphs in HBM; a trace of histo / ig / triangle requests replayed
in real time with continuous batching into the persistent queue kernel.

    from bale_old_gb300 import serve
    with serve.Server() as s:
        t = s.add_table(table)            # numpy int64
        c = s.add_counts(1 << 20)
        g = s.add_graph(L)                # SparseMatrix
        reqs = [serve.ig(t, index, out, arrival=0.0), serve.histo(c, updates, arrival=0.001),
                serve.triangles(g, out1, arrival=0.002)]
        latency, stats = s.run(reqs)

Host arrays must stay alive until run() returns; pinned arrays (e.g. from
torch's pin_memory) let the copies overlap the GPU work.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import BaleError, SparseMatrix, _last_error, _lib
from ._lib import P64, bale_request_t, bale_serve_stats_t

HISTO, IG, TRIANGLES = 0, 1, 2


@dataclass
class Request:
    kind: int
    obj: int
    index: np.ndarray | None
    out: np.ndarray | None
    arrival: float
    shift: int = 0


def ig(obj: int, index: np.ndarray, out: np.ndarray, arrival: float = 0.0, shift: int = 0) -> Request:
    if out.size < index.size:
        raise ValueError("out is shorter than the request")
    return Request(IG, obj, index, out, arrival, shift)


def histo(obj: int, index: np.ndarray, arrival: float = 0.0, shift: int = 0) -> Request:
    return Request(HISTO, obj, index, None, arrival, shift)


def triangles(obj: int, out: np.ndarray, arrival: float = 0.0) -> Request:
    if out.size < 1:
        raise ValueError("out needs one int64")
    return Request(TRIANGLES, obj, None, out, arrival)


def _ptr(a):
    return None if a is None else a.ctypes.data


def _check(a, name):
    if a is not None and (not isinstance(a, np.ndarray) or a.dtype != np.int64 or not a.flags.c_contiguous):
        raise TypeError(f"{name} must be a C-contiguous numpy int64 array")


class Server:
    def __init__(self, arena_bytes: int = 0, max_active: int = 64):
        h = _lib.bale_server_create(int(arena_bytes), int(max_active))
        if not h:
            raise BaleError(f"bale_server_create: {_last_error()}")
        self._h = h
        self._counts: dict[int, int] = {}

    def _obj(self, rc: int, what: str) -> int:
        if rc < 0:
            raise BaleError(f"{what}: status {-rc}: {_last_error()}")
        return rc

    def add_table(self, table: np.ndarray) -> int:
        _check(table, "table")
        return self._obj(_lib.bale_server_add_table(self._h, table.ctypes.data_as(P64), table.size), "add_table")

    def add_counts(self, ncounts: int) -> int:
        obj = self._obj(_lib.bale_server_add_counts(self._h, int(ncounts)), "add_counts")
        self._counts[obj] = int(ncounts)
        return obj

    def add_graph(self, L: SparseMatrix) -> int:
        return self._obj(_lib.bale_server_add_graph(self._h, L.offset.ctypes.data_as(P64),
                                                    L.nonzero.ctypes.data_as(P64), L.numrows, L.nnz), "add_graph")

    def read_counts(self, obj: int) -> np.ndarray:
        out = np.zeros(self._counts[obj], np.int64)
        if _lib.bale_server_read_counts(self._h, obj, out.ctypes.data_as(P64), out.size) != 0:
            raise BaleError(f"read_counts: {_last_error()}")
        return out

    def run(self, requests: list[Request]) -> tuple[np.ndarray, dict]:
        arr = (bale_request_t * max(1, len(requests)))()
        for k, r in enumerate(requests):
            _check(r.index, "index")
            _check(r.out, "out")
            n = 0 if r.index is None else r.index.size
            arr[k] = bale_request_t(r.kind, r.obj, r.shift, 0, n, _ptr(r.index), _ptr(r.out), float(r.arrival))
        lat = np.zeros(max(1, len(requests)), np.float64)
        st = bale_serve_stats_t()
        rc = _lib.bale_server_run(self._h, arr, len(requests), lat.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.byref(st))
        if rc != 0:
            raise BaleError(f"bale_server_run: status {rc}: {_last_error()}")
        stats = {f: getattr(st, f) for f, _ in bale_serve_stats_t._fields_}
        return lat[: len(requests)], stats

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.bale_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def poisson_arrivals(n: int, rate_per_s: float, seed: int) -> np.ndarray:
    """Arrival times (seconds) of a Poisson process of the given rate."""
    if rate_per_s <= 0:
        return np.zeros(n)
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_per_s, size=n))
