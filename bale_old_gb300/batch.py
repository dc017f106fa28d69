"""Batched execution: many histo / ig / triangle instances in one CUDA graph
(bale_batch_* in include/bale_gb300.h).

    from bale_old_gb300 import batch
    b = batch.Batch([batch.histo(counts, index), batch.ig(tgt, index, table),
                     batch.triangles(offset, nonzero, count)])
    b.run()            # asynchronous on the current stream; replay at will
    b.bad()            # per-instance out-of-range / malformed counts of the last run

All tensors are CUDA int64 tensors and must stay alive while the batch exists
(the batch keeps references).  Results equal the per-instance entry points:
histo adds into counts, ig overwrites tgt, triangles add into count[0].
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import BaleError, _dptr, _last_error, _lib, _stream
from ._lib import bale_instance_t

HISTO, IG, TRIANGLES = 0, 1, 2
STAT_NAMES = ("tasks", "tasks_histo_smem", "tasks_histo_l2", "tasks_ig", "tasks_tri_light", "tasks_tri_heavy",
              "standalone_instances", "instances", "side_streams")


@dataclass
class Instance:
    kind: int
    shift: int
    n: int
    m: int
    out: object
    inp: object
    aux: object

    def struct(self) -> bale_instance_t:
        aux = _dptr(self.aux, "aux") if self.aux is not None else None
        return bale_instance_t(self.kind, self.shift, self.n, self.m, _dptr(self.out, "out"),
                               _dptr(self.inp, "in") if self.n > 0 or self.kind == TRIANGLES else None, aux)


def histo(counts, index, shift: int = 0) -> Instance:
    return Instance(HISTO, shift, index.numel(), counts.numel(), counts, index, None)


def ig(tgt, index, table, shift: int = 0) -> Instance:
    if tgt.numel() < index.numel():
        raise ValueError("tgt is shorter than the request count")
    return Instance(IG, shift, index.numel(), table.numel(), tgt, index, table)


def triangles(offset, nonzero, count) -> Instance:
    return Instance(TRIANGLES, 0, offset.numel() - 1, nonzero.numel(), count, offset, nonzero)


class Batch:
    def __init__(self, instances: Sequence[Instance]):
        self._inst = list(instances)
        arr = (bale_instance_t * max(1, len(self._inst)))(*[x.struct() for x in self._inst])
        h = _lib.bale_batch_create(arr, len(self._inst))
        if not h:
            raise BaleError(f"bale_batch_create: {_last_error()}")
        self._h = h

    def run(self, stream=None) -> None:
        if _lib.bale_batch_run(self._h, _stream(stream)) != 0:
            raise BaleError(f"bale_batch_run: {_last_error()}")

    def bad(self) -> np.ndarray:
        out = np.zeros(max(1, len(self._inst)), np.int64)
        if _lib.bale_batch_bad(self._h, out.ctypes.data_as(C.POINTER(C.c_int64)), len(self._inst)) != 0:
            raise BaleError(f"bale_batch_bad: {_last_error()}")
        return out[: len(self._inst)]

    def stats(self) -> dict[str, int]:
        out = np.zeros(len(STAT_NAMES), np.int64)
        _lib.bale_batch_stats(self._h, out.ctypes.data_as(C.POINTER(C.c_int64)), out.size)
        return dict(zip(STAT_NAMES, out.tolist()))

    def plan(self) -> np.ndarray:
        """Per instance: the side stream it runs on as its own kernels, or -1
        for the work queue."""
        out = np.zeros(max(1, len(self._inst)), np.int64)
        if _lib.bale_batch_plan(self._h, out.ctypes.data_as(C.POINTER(C.c_int64)), len(self._inst)) != 0:
            raise BaleError(f"bale_batch_plan: {_last_error()}")
        return out[: len(self._inst)]

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.bale_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
