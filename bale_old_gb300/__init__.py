"""bale_old_gb300 -- bale's irregular-access core (histo, ig, triangles) on one
GB300 (sm_103a), behind the reference's own entry points.

The compute is in libbale_gb300.so (hand-written CUDA + host C, C ABI in
include/bale_gb300.h).  This module is the host-side mirror of the reference
interface for Python callers: the same names as the reference's apps
(histo_agi, ig_exstack, triangle_agi, ...), the same argument meaning
(histo ADDS into counts, ig OVERWRITES tgt, triangles return the count and a
work tally), the same return value (wall seconds).  Where the reference
returns -1.0 for a failure, these raise BaleError with the library's message.
There is no CPU path: every call goes through the CUDA library, and importing
the package fails if the library is not built.
"""
from __future__ import annotations

import ctypes as C
from typing import Iterable, Optional, Sequence

import numpy as np

from ._lib import LIB_PATH, P64, PSM, load, sparsemat_t

__all__ = [
    "BaleError", "SparseMatrix", "LIB_PATH",
    "histo_agi", "histo_exstack", "histo_exstack2", "histo_conveyor",
    "ig_agi", "ig_exstack", "ig_exstack2", "ig_conveyor",
    "triangle_agi", "triangle_exstack_push", "triangle_exstack2_push",
    "triangle_convey_push", "triangle_agi_iter",
    "histo_dev", "ig_dev", "triangle_dev", "ig_dev_noalloc", "TrianglePrepared", "l2_red_rate",
    "graph_build_dev", "gen_rmat_dev", "transpose_dev", "permute_dev", "rand_perm_dev", "rand_perm_exstack_dev", "rand_perm_exstack2_dev",
    "write_matrix_mm", "mm_header", "read_matrix_mm_dev",
    "write_sparse_matrix", "write_sparse_matrix_dev", "sparse_matrix_header", "read_sparse_matrix_dev",
    "splitmix64", "gen_uniform", "gen_values", "gen_uniform_dev", "gen_values_dev", "gen_negative_table", "gen_zipf",
    "keyed_perm", "gen_rmat", "gen_erdos_renyi", "gen_kronecker", "kronecker_triangles",
    "set_host_threads", "release_buffers", "version", "pack_index",
    "tune_set", "tune_get", "tune_knobs", "device_caps",
]

_lib = load()


class BaleError(RuntimeError):
    """A drop-in returned -1.0 or a device entry point returned a status."""


def _last_error() -> str:
    msg = _lib.bale_last_error()
    return msg.decode() if msg else ""


def _arr(a: np.ndarray, name: str, writable: bool = False) -> np.ndarray:
    if not isinstance(a, np.ndarray) or a.dtype != np.int64 or not a.flags.c_contiguous:
        raise TypeError(f"{name} must be a C-contiguous numpy int64 array")
    if writable and not a.flags.writeable:
        raise ValueError(f"{name} must be writable")
    return a


def _p(a: np.ndarray):
    return a.ctypes.data_as(P64)


def _seconds(t: float, what: str) -> float:
    if t < 0:
        raise BaleError(f"{what}: {_last_error()}")
    return t


def pack_index(index: np.ndarray) -> np.ndarray:
    """The reference's packed index for one PE: (index << 16) | 0
    (apps/histo_src/histo.upc:150, apps/ig_src/ig.upc:174)."""
    return (np.asarray(index, dtype=np.int64) << 16).astype(np.int64)


# --------------------------------------------------------------------------
# sparse matrices
# --------------------------------------------------------------------------
class SparseMatrix:
    """A one-PE sparsemat_t whose arrays are numpy int64 buffers:
    ``offset`` (numrows+1 row offsets) and ``nonzero`` (ascending columns)."""

    def __init__(self, offset: np.ndarray, nonzero: np.ndarray, numcols: Optional[int] = None):
        self.offset = np.ascontiguousarray(offset, dtype=np.int64)
        self.nonzero = np.ascontiguousarray(nonzero, dtype=np.int64)
        n = int(self.offset.shape[0]) - 1
        if n < 0:
            raise ValueError("offset needs at least one entry")
        self.numrows = n
        self.numcols = n if numcols is None else int(numcols)
        nnz = int(self.nonzero.shape[0])
        po, pn = _p(self.offset), _p(self.nonzero)
        self._struct = sparsemat_t(0, n, n, self.numcols, nnz, nnz, po, po, pn, pn)

    @property
    def nnz(self) -> int:
        return int(self.nonzero.shape[0])

    @property
    def struct(self) -> sparsemat_t:
        return self._struct

    def ptr(self):
        return C.pointer(self._struct)

    @classmethod
    def _from_c(cls, m, what: str) -> "SparseMatrix":
        if not m:
            raise BaleError(f"{what}: generator failed (bad parameters or out of memory)")
        try:
            s = m.contents
            n, nnz = int(s.numrows), int(s.nnz)
            off = np.ctypeslib.as_array(s.loffset, shape=(n + 1,)).copy()
            col = (np.ctypeslib.as_array(s.lnonzero, shape=(nnz,)).copy() if nnz
                   else np.zeros(0, np.int64))
            return cls(off, col, int(s.numcols))
        finally:
            _lib.bale_free_matrix(m)

    def row(self, i: int) -> np.ndarray:
        return self.nonzero[self.offset[i]:self.offset[i + 1]]


# --------------------------------------------------------------------------
# drop-ins: histogram (apps/histo_src/histo.h:47-50)
# --------------------------------------------------------------------------
def histo_agi(index: np.ndarray, counts: np.ndarray, length: Optional[int] = None) -> float:
    """counts[index[i]] += 1 for i < length (default len(index))."""
    _arr(index, "index"), _arr(counts, "counts", True)
    n = index.size if length is None else int(length)
    return _seconds(_lib.histo_agi(_p(index), n, _p(counts)), "histo_agi")


def histo_exstack(pckindx: np.ndarray, lcounts: np.ndarray, buf_cnt: int = 1024,
                  length: Optional[int] = None) -> float:
    """lcounts[pckindx[i] >> 16] += 1 (one PE)."""
    _arr(pckindx, "pckindx"), _arr(lcounts, "lcounts", True)
    n = pckindx.size if length is None else int(length)
    return _seconds(_lib.histo_exstack(_p(pckindx), n, _p(lcounts), buf_cnt), "histo_exstack")


def histo_exstack2(pckindx: np.ndarray, lcounts: np.ndarray, buf_cnt: int = 1024,
                   length: Optional[int] = None) -> float:
    _arr(pckindx, "pckindx"), _arr(lcounts, "lcounts", True)
    n = pckindx.size if length is None else int(length)
    return _seconds(_lib.histo_exstack2(_p(pckindx), n, _p(lcounts), buf_cnt), "histo_exstack2")


def histo_conveyor(pckindx: np.ndarray, lcounts: np.ndarray, length: Optional[int] = None) -> float:
    _arr(pckindx, "pckindx"), _arr(lcounts, "lcounts", True)
    n = pckindx.size if length is None else int(length)
    return _seconds(_lib.histo_conveyor(_p(pckindx), n, _p(lcounts)), "histo_conveyor")


# --------------------------------------------------------------------------
# drop-ins: index gather (apps/ig_src/ig.h:49-52)
# --------------------------------------------------------------------------
def ig_agi(tgt: np.ndarray, index: np.ndarray, table: np.ndarray, length: Optional[int] = None) -> float:
    """tgt[i] = table[index[i]] for i < length (default len(index))."""
    _arr(tgt, "tgt", True), _arr(index, "index"), _arr(table, "table")
    n = index.size if length is None else int(length)
    if tgt.size < n:
        raise ValueError("tgt is shorter than the request count")
    return _seconds(_lib.ig_agi(_p(tgt), _p(index), n, _p(table)), "ig_agi")


def ig_exstack(tgt: np.ndarray, pckindx: np.ndarray, ltable: np.ndarray, buf_cnt: int = 1024,
               length: Optional[int] = None) -> float:
    """tgt[i] = ltable[pckindx[i] >> 16] (one PE)."""
    _arr(tgt, "tgt", True), _arr(pckindx, "pckindx"), _arr(ltable, "ltable")
    n = pckindx.size if length is None else int(length)
    if tgt.size < n:
        raise ValueError("tgt is shorter than the request count")
    return _seconds(_lib.ig_exstack(_p(tgt), _p(pckindx), n, _p(ltable), buf_cnt), "ig_exstack")


def ig_exstack2(tgt: np.ndarray, pckindx: np.ndarray, ltable: np.ndarray, buf_cnt: int = 1024,
                length: Optional[int] = None) -> float:
    _arr(tgt, "tgt", True), _arr(pckindx, "pckindx"), _arr(ltable, "ltable")
    n = pckindx.size if length is None else int(length)
    if tgt.size < n:
        raise ValueError("tgt is shorter than the request count")
    return _seconds(_lib.ig_exstack2(_p(tgt), _p(pckindx), n, _p(ltable), buf_cnt), "ig_exstack2")


def ig_conveyor(tgt: np.ndarray, pckindx: np.ndarray, ltable: np.ndarray,
                length: Optional[int] = None) -> float:
    _arr(tgt, "tgt", True), _arr(pckindx, "pckindx"), _arr(ltable, "ltable")
    n = pckindx.size if length is None else int(length)
    if tgt.size < n:
        raise ValueError("tgt is shorter than the request count")
    return _seconds(_lib.ig_conveyor(_p(tgt), _p(pckindx), n, _p(ltable)), "ig_conveyor")


# --------------------------------------------------------------------------
# drop-ins: triangles (apps/triangle_src/triangle.h:50-61)
# --------------------------------------------------------------------------
def _tri(fn, name: str, L: SparseMatrix, U: Optional[SparseMatrix], alg: int, *extra):
    if not isinstance(L, SparseMatrix):
        raise TypeError("L must be a SparseMatrix")
    cnt, sr = C.c_int64(0), C.c_int64(0)
    u = U.ptr() if U is not None else None
    t = fn(C.byref(cnt), C.byref(sr), L.ptr(), u, alg, *extra)
    return int(cnt.value), int(sr.value), _seconds(t, name)


def triangle_agi(L: SparseMatrix, U: Optional[SparseMatrix] = None, alg: int = 0):
    """(count, sr, seconds).  alg 0: the triangles of the strictly lower tidy
    L; any other alg: the reference's alg 1, the sum over L's nonzeros (i,j)
    of |U_i and U_j| for the strictly upper tidy U (required), which is the
    same count when U is L's transpose."""
    return _tri(_lib.triangle_agi, "triangle_agi", L, U, alg)


def triangle_exstack_push(L: SparseMatrix, U: Optional[SparseMatrix] = None, alg: int = 0,
                          bufsiz: int = 1024):
    return _tri(_lib.triangle_exstack_push, "triangle_exstack_push", L, U, alg, bufsiz)


def triangle_exstack2_push(L: SparseMatrix, U: Optional[SparseMatrix] = None, alg: int = 0,
                           bufsiz: int = 1024):
    return _tri(_lib.triangle_exstack2_push, "triangle_exstack2_push", L, U, alg, bufsiz)


def triangle_convey_push(L: SparseMatrix, U: Optional[SparseMatrix] = None, alg: int = 0):
    return _tri(_lib.triangle_convey_push, "triangle_convey_push", L, U, alg)


def triangle_agi_iter(L: SparseMatrix, U: Optional[SparseMatrix] = None, alg: int = 0):
    return _tri(_lib.triangle_agi_iter, "triangle_agi_iter", L, U, alg)


# --------------------------------------------------------------------------
# device-resident entry points (torch CUDA tensors as plumbing)
# --------------------------------------------------------------------------
def _dptr(t, name: str, dtype=None) -> int:
    import torch

    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != torch.int64 or not t.is_contiguous():
        raise TypeError(f"{name} must be a contiguous int64 tensor")
    return t.data_ptr()


def _stream(stream) -> int:
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream
    return int(getattr(stream, "cuda_stream", stream))


def _status(rc: int, what: str) -> None:
    if rc != 0:
        raise BaleError(f"{what}: status {rc}: {_last_error()}")


def histo_dev(counts, index, shift: int = 0, bad=None, stream=None, n: Optional[int] = None) -> None:
    """counts[index[i] >> shift] += 1 on the device (asynchronous)."""
    nn = index.numel() if n is None else int(n)
    _status(_lib.bale_histo_dev(_dptr(counts, "counts"), counts.numel(), _dptr(index, "index"), nn,
                                shift, _dptr(bad, "bad") if bad is not None else None,
                                _stream(stream)), "bale_histo_dev")


def ig_dev(tgt, index, table, shift: int = 0, bad=None, stream=None, n: Optional[int] = None) -> None:
    """tgt[i] = table[index[i] >> shift] on the device (asynchronous)."""
    nn = index.numel() if n is None else int(n)
    _status(_lib.bale_ig_dev(_dptr(tgt, "tgt"), _dptr(index, "index"), nn, _dptr(table, "table"),
                             table.numel(), shift, _dptr(bad, "bad") if bad is not None else None,
                             _stream(stream)), "bale_ig_dev")


def ig_dev_noalloc(tgt, index, table, shift: int = 0, bad=None, stream=None,
                   n: Optional[int] = None) -> None:
    """Same result as ig_dev, for callers that cannot allocate device memory:
    the scratch is a fixed array inside the library (at most 262144 requests
    per call; tgt and index 16-byte aligned).  Calls share that array, so
    calls that overlap on the GPU must be serialised by the caller."""
    nn = index.numel() if n is None else int(n)
    _status(_lib.bale_ig_dev_noalloc(_dptr(tgt, "tgt"), _dptr(index, "index"), nn, _dptr(table, "table"),
                                     table.numel(), shift, _dptr(bad, "bad") if bad is not None else None,
                                     _stream(stream)), "bale_ig_dev_noalloc")


def triangle_dev(offset, nonzero, count, work=None, bad=None, stream=None) -> None:
    """count[0] += triangles of the device CSR (asynchronous)."""
    _status(_lib.bale_triangle_dev(_dptr(offset, "offset"), _dptr(nonzero, "nonzero"),
                                   offset.numel() - 1, nonzero.numel(), _dptr(count, "count"),
                                   _dptr(work, "work") if work is not None else None,
                                   _dptr(bad, "bad") if bad is not None else None,
                                   _stream(stream)), "bale_triangle_dev")


def l2_red_rate(counts, n: int, stream=None) -> None:
    """n +1 reductions at hashed positions of counts (device int64): the L2
    reduction-rate probe that bounds a histogram whose table fits in L2."""
    _status(_lib.bale_l2_red_rate(_dptr(counts, "counts"), counts.numel(), int(n), _stream(stream)),
            "bale_l2_red_rate")


def graph_build_dev(u, v, n: int, stream=None):
    """Degree-ordered strictly lower CSR of the undirected edges (u[e], v[e])
    (device int64 tensors) on n vertices, built on the device: returns
    (offset, nonzero) device tensors, nonzero trimmed to nnz."""
    import torch

    m = u.numel()
    if v.numel() != m:
        raise ValueError("u and v differ in length")
    off = torch.empty(n + 1, dtype=torch.int64, device=u.device)
    nz = torch.empty(max(m, 1), dtype=torch.int64, device=u.device)
    nnz = C.c_int64(0)
    _status(_lib.bale_graph_build_dev(_dptr(u, "u") if m else None, _dptr(v, "v") if m else None, m, int(n),
                                      _dptr(off, "offset"), _dptr(nz, "nonzero"), C.byref(nnz), _stream(stream)),
            "bale_graph_build_dev")
    return off, nz[: nnz.value]


def gen_rmat_dev(scale: int, edgefactor: int, a: float, b: float, c: float, seed: int, device=None, stream=None):
    """gen_rmat's graph generated and built on the device (bit-identical):
    returns (offset, nonzero) device int64 tensors."""
    import torch

    dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    n = 1 << scale
    off = torch.empty(n + 1, dtype=torch.int64, device=dev)
    nz = torch.empty(edgefactor * n, dtype=torch.int64, device=dev)
    nnz = C.c_int64(0)
    _status(_lib.bale_gen_rmat_dev(scale, edgefactor, a, b, c, seed & (2**64 - 1), _dptr(off, "offset"),
                                   _dptr(nz, "nonzero"), C.byref(nnz), _stream(stream)), "bale_gen_rmat_dev")
    return off, nz[: nnz.value]


def transpose_dev(offset, nonzero, numcols: int, stream=None):
    """spmat's transpose_matrix_agi on the device: returns At's (offset, nonzero)."""
    import torch

    n, nnz = offset.numel() - 1, nonzero.numel()
    toff = torch.empty(numcols + 1, dtype=torch.int64, device=offset.device)
    tcol = torch.empty(max(nnz, 1), dtype=torch.int64, device=offset.device)
    _status(_lib.bale_transpose_dev(_dptr(offset, "offset"), _dptr(nonzero, "nonzero") if nnz else None, n,
                                    int(numcols), nnz, _dptr(toff, "toffset"), _dptr(tcol, "tnonzero"),
                                    _stream(stream)), "bale_transpose_dev")
    return toff, tcol[:nnz]


def permute_dev(offset, nonzero, numcols: int, rperminv, cperminv, stream=None):
    """spmat's permute_matrix_agi on the device: returns (offset, nonzero)."""
    import torch

    n, nnz = offset.numel() - 1, nonzero.numel()
    poff = torch.empty(n + 1, dtype=torch.int64, device=offset.device)
    pcol = torch.empty(max(nnz, 1), dtype=torch.int64, device=offset.device)
    _status(_lib.bale_permute_dev(_dptr(offset, "offset"), _dptr(nonzero, "nonzero") if nnz else None, n,
                                  int(numcols), nnz, _dptr(rperminv, "rperminv"), _dptr(cperminv, "cperminv"),
                                  _dptr(poff, "poffset"), _dptr(pcol, "pnonzero"), _stream(stream)),
            "bale_permute_dev")
    return poff, pcol[:nnz]


def rand_perm_dev(n: int, seed: int, device=None, stream=None):
    """spmat's rand_permp_agi(n, seed) on the device (a device int64 tensor).
    Seed 0 continues the C library's drand48 stream; every call leaves that
    stream past the reference's last draw."""
    import torch

    dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    out = torch.empty(max(n, 1), dtype=torch.int64, device=dev)
    _status(_lib.bale_rand_perm_dev(int(n), seed & (2**64 - 1), _dptr(out, "perm"), _stream(stream)),
            "bale_rand_perm_dev")
    return out[:n]


def rand_perm_exstack_dev(n: int, seed: int, buf_cnt: int = 1024, device=None, stream=None):
    """spmat's rand_permp_exstack(n, seed, buf_cnt) on the device (a device
    int64 tensor); the default buf_cnt gives rand_permp(n, seed)."""
    import torch

    dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    out = torch.empty(max(n, 1), dtype=torch.int64, device=dev)
    _status(_lib.bale_rand_perm_exstack_dev(int(n), seed & (2**64 - 1), int(buf_cnt), _dptr(out, "perm"),
                                            _stream(stream)), "bale_rand_perm_exstack_dev")
    return out[:n]


def rand_perm_exstack2_dev(n: int, seed: int, buf_cnt: int = 1024, device=None, stream=None):
    """spmat's rand_permp_exstack2(n, seed, buf_cnt) on the device, which in
    the reference is rand_permp_exstack(n, seed, buf_cnt)."""
    import torch

    dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    out = torch.empty(max(n, 1), dtype=torch.int64, device=dev)
    _status(_lib.bale_rand_perm_exstack2_dev(int(n), seed & (2**64 - 1), int(buf_cnt), _dptr(out, "perm"),
                                             _stream(stream)), "bale_rand_perm_exstack2_dev")
    return out[:n]


def write_matrix_mm(L: "SparseMatrix", path) -> None:
    """spmat's write_matrix_mm: the matrix as a MatrixMarket pattern file."""
    _status(_lib.bale_write_matrix_mm(L.ptr(), str(path).encode()), "bale_write_matrix_mm")


def mm_header(path) -> tuple[int, int, int, int]:
    """(numrows, numcols, nnz, fields) of a MatrixMarket coordinate file."""
    nr, nc, nnz, body, fields = C.c_int64(0), C.c_int64(0), C.c_int64(0), C.c_int64(0), C.c_int(0)
    _status(_lib.bale_mm_header(str(path).encode(), C.byref(nr), C.byref(nc), C.byref(nnz), C.byref(body),
                                C.byref(fields)), "bale_mm_header")
    return nr.value, nc.value, nnz.value, fields.value


def read_matrix_mm_dev(path, device=None, stream=None):
    """spmat's read_matrix_mm_to_dist at one PE, parsed on the device:
    returns (offset, nonzero, numcols) with device int64 tensors."""
    import torch

    nr, nc, nnz, _ = mm_header(path)
    dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    off = torch.empty(nr + 1, dtype=torch.int64, device=dev)
    col = torch.empty(max(nnz, 1), dtype=torch.int64, device=dev)
    _status(_lib.bale_read_matrix_mm_dev(str(path).encode(), _dptr(off, "offset"), _dptr(col, "nonzero"),
                                         _stream(stream)), "bale_read_matrix_mm_dev")
    return off, col[:nnz], nc


def write_sparse_matrix(L: "SparseMatrix", dirname) -> None:
    """spmat's write_sparse_matrix_agi at one PE: the matrix as a binary
    dataset directory (metadata, rowcnt_0, nonzero_0)."""
    _status(_lib.bale_write_sparse_matrix(str(dirname).encode(), L.ptr()), "bale_write_sparse_matrix")


def write_sparse_matrix_dev(dirname, offset, nonzero, numcols: int, nwriters: int = 1, stream=None) -> None:
    """A device CSR written as a binary dataset with nwriters row blocks (the
    layout the reference writes at nwriters PEs)."""
    nnz = nonzero.numel()
    _status(_lib.bale_write_sparse_matrix_dev(str(dirname).encode(), _dptr(offset, "offset"),
                                              _dptr(nonzero, "nonzero") if nnz else None, offset.numel() - 1,
                                              int(numcols), nnz, int(nwriters), _stream(stream)),
            "bale_write_sparse_matrix_dev")


def sparse_matrix_header(dirname) -> tuple[int, int, int, int]:
    """(numrows, numcols, nnz, nwriters) of a binary dataset."""
    v = [C.c_int64(0) for _ in range(4)]
    _status(_lib.bale_sparse_matrix_header(str(dirname).encode(), *(C.byref(x) for x in v)),
            "bale_sparse_matrix_header")
    return tuple(x.value for x in v)


def read_sparse_matrix_dev(dirname, device=None, stream=None):
    """A binary dataset (any number of writers) read into device int64
    tensors: returns (offset, nonzero, numcols)."""
    import torch

    nr, nc, nnz, _ = sparse_matrix_header(dirname)
    dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    off = torch.empty(nr + 1, dtype=torch.int64, device=dev)
    col = torch.empty(max(nnz, 1), dtype=torch.int64, device=dev)
    _status(_lib.bale_read_sparse_matrix_dev(str(dirname).encode(), _dptr(off, "offset"), _dptr(col, "nonzero"),
                                             _stream(stream)), "bale_read_sparse_matrix_dev")
    return off, col[:nnz], nc


class TrianglePrepared:
    """A device CSR counted repeatedly (bale_triangle_prepare): validation,
    the 32-bit column copy and the transpose are built once; count() adds
    the triangle count into a device int64 each call.  offset/nonzero must
    stay alive and unchanged until close()."""

    def __init__(self, offset, nonzero, bad=None, stream=None):
        self._keep = (offset, nonzero)
        h = _lib.bale_triangle_prepare(_dptr(offset, "offset"), _dptr(nonzero, "nonzero"), offset.numel() - 1,
                                       nonzero.numel(), _dptr(bad, "bad") if bad is not None else None,
                                       _stream(stream))
        if not h:
            raise BaleError(f"bale_triangle_prepare: {_last_error()}")
        self._h = h

    def count(self, count, work=None, stream=None) -> None:
        _status(_lib.bale_triangle_count_prepared(self._h, _dptr(count, "count"),
                                                  _dptr(work, "work") if work is not None else None,
                                                  _stream(stream)), "bale_triangle_count_prepared")

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.bale_triangle_release(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# --------------------------------------------------------------------------
# seeded inputs (include/bale_inputs.h)
# --------------------------------------------------------------------------
def splitmix64(seed: int, i: int) -> int:
    return int(_lib.bale_splitmix64(seed & (2**64 - 1), i))


def _gen_status(rc: int, what: str) -> None:
    if rc != 0:
        raise BaleError(f"{what}: invalid parameters")


def gen_uniform(n: int, rng: int, seed: int, packed: bool = False) -> np.ndarray:
    out = np.empty(n, np.int64)
    _gen_status(_lib.bale_gen_uniform(_p(out), n, rng, seed & (2**64 - 1), int(packed)), "gen_uniform")
    return out


def gen_uniform_dev(out, rng: int, seed: int, packed: bool = False, stream=None) -> None:
    """gen_uniform into a device int64 tensor (same bits as the host one)."""
    _status(_lib.bale_gen_uniform_dev(_dptr(out, "out"), out.numel(), rng, seed & (2**64 - 1), int(packed),
                                      _stream(stream)), "bale_gen_uniform_dev")


def gen_values_dev(out, seed: int, stream=None) -> None:
    """gen_values into a device int64 tensor (same bits as the host one)."""
    _status(_lib.bale_gen_values_dev(_dptr(out, "out"), out.numel(), seed & (2**64 - 1), _stream(stream)),
            "bale_gen_values_dev")


def gen_values(n: int, seed: int) -> np.ndarray:
    out = np.empty(n, np.int64)
    _gen_status(_lib.bale_gen_values(_p(out), n, seed & (2**64 - 1)), "gen_values")
    return out


def gen_negative_table(n: int) -> np.ndarray:
    out = np.empty(n, np.int64)
    _gen_status(_lib.bale_gen_negative_table(_p(out), n), "gen_negative_table")
    return out


def gen_zipf(n: int, rng: int, s: float, seed_rank: int, seed_perm: int,
             packed: bool = False) -> np.ndarray:
    out = np.empty(n, np.int64)
    _gen_status(_lib.bale_gen_zipf(_p(out), n, rng, s, seed_rank & (2**64 - 1),
                                   seed_perm & (2**64 - 1), int(packed)), "gen_zipf")
    return out


def keyed_perm(r: int, rng: int, key: int) -> int:
    return int(_lib.bale_keyed_perm(r, rng, key & (2**64 - 1)))


def gen_rmat(scale: int, edgefactor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 6) -> SparseMatrix:
    return SparseMatrix._from_c(_lib.bale_gen_rmat(scale, edgefactor, a, b, c, seed & (2**64 - 1)),
                                "gen_rmat")


def gen_erdos_renyi(n: int, p: float, seed: int = 7) -> SparseMatrix:
    return SparseMatrix._from_c(_lib.bale_gen_erdos_renyi(n, p, seed & (2**64 - 1)), "gen_erdos_renyi")


def gen_kronecker(mode: int, specs: Sequence[int]) -> SparseMatrix:
    arr = np.ascontiguousarray(np.asarray(list(specs), dtype=np.int64))
    return SparseMatrix._from_c(_lib.bale_gen_kronecker(mode, _p(arr), arr.size), "gen_kronecker")


def kronecker_triangles(mode: int, specs: Iterable[int]) -> int:
    arr = np.ascontiguousarray(np.asarray(list(specs), dtype=np.int64))
    return int(_lib.bale_kronecker_triangles(mode, _p(arr), arr.size))


def tune_set(name: str, value: int) -> None:
    """Pin a launch knob (e.g. "ig.unroll"); -1 returns it to automatic."""
    if _lib.bale_tune_set(name.encode(), int(value)) != 0:
        raise BaleError(_last_error())


def tune_get(name: str) -> int:
    v = int(_lib.bale_tune_get(name.encode()))
    if v == -2:
        raise BaleError(f"unknown tuning knob {name!r}")
    return v


def tune_knobs() -> dict[str, int]:
    return {(_lib.bale_tune_name(i)).decode(): tune_get(_lib.bale_tune_name(i).decode())
            for i in range(_lib.bale_tune_count())}


def set_host_threads(n: int) -> None:
    _lib.bale_set_host_threads(int(n))


def release_buffers() -> None:
    _lib.bale_release_buffers()


CAP_NAMES = ("sms", "pageable_memory_access", "pageable_uses_host_page_tables", "concurrent_managed_access",
             "l2_bytes", "smem_optin_per_block", "host_pointer_for_registered_mem", "copy_engines",
             "unified_addressing")


def device_caps() -> dict[str, int]:
    """Facts about the current CUDA device (bale_device_caps)."""
    out = np.zeros(len(CAP_NAMES), np.int64)
    if _lib.bale_device_caps(_p(out), out.size) != 0:
        raise BaleError(_last_error())
    return dict(zip(CAP_NAMES, out.tolist()))


def version() -> str:
    return _lib.bale_version().decode()


def _apply_committed_tuning() -> None:
    """Apply bale_old_gb300/tuning/gb300.tune (autotuner output) if present."""
    from pathlib import Path

    p = Path(__file__).resolve().parent / "tuning" / "gb300.tune"
    if p.exists():
        _lib.bale_tune_load(str(p).encode())


_apply_committed_tuning()
