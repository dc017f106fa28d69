"""ctypes access to the parity checker -- TEST INFRASTRUCTURE ONLY.

Two libraries, both built by oracle/Makefile:

* ``_build/liboracle.so`` -- the C restatement in bale_oracle.c (always
  buildable: plain gcc, no reference tree needed).  Used by tests/ as the
  checker and by bench.py as the timed CPU baseline.
* ``_ref/libbale_ref.so`` -- the reference's own unmodified SHMEM-mode sources
  compiled against the single-PE shim.  Only exists where the reference tree
  is present; it pins the restatement (tests/golden/make_golden.py).

Nothing in the shipped package imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libbale_ref.so"
# The reference tree: $BALE_REFERENCE_TREE, else a directory named
# "reference" beside this repository's root.
REF_TREE = Path(os.environ.get("BALE_REFERENCE_TREE") or HERE.parent.parent / "reference")

i64 = C.c_int64
P64 = C.POINTER(C.c_int64)


def _p(a: np.ndarray):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(P64)


def build_port() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    return PORT_LIB


def build_ref() -> Path | None:
    """Compile the reference's sources into _ref/ when the tree is present."""
    if not (REF_TREE / "apps" / "histo_src" / "histo_agi.upc").exists():
        return None
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REF_TREE}"], check=True)
    return REF_LIB


class Oracle:
    """The C restatement (bale_oracle.c)."""

    def __init__(self, path: Path | None = None):
        if path is None:
            path = PORT_LIB if PORT_LIB.exists() else build_port()
        lib = C.CDLL(str(path))
        sig = {
            "orc_histo_agi": (None, [P64, i64, P64]),
            "orc_histo_exstack": (None, [P64, i64, P64]),
            "orc_ig_agi": (None, [P64, P64, i64, P64]),
            "orc_ig_exstack": (None, [P64, P64, i64, P64]),
            "orc_triangle_agi": (i64, [P64, P64, i64, P64]),
            "orc_triangle_exstack_push": (i64, [P64, P64, i64, P64]),
            "orc_triangle_work": (None, [P64, P64, i64, P64, P64]),
            "orc_is_strict_lower_tidy": (C.c_int, [P64, P64, i64]),
            "orc_histo_agi_mt": (None, [P64, i64, P64, C.c_int]),
            "orc_ig_agi_mt": (None, [P64, P64, i64, P64, C.c_int]),
            "orc_triangle_agi_mt": (i64, [P64, P64, i64, C.c_int]),
            "orc_transpose": (C.c_int, [P64, P64, i64, i64, P64, P64]),
            "orc_permute": (None, [P64, P64, i64, P64, P64, P64, P64]),
            "orc_rand_perm": (C.c_int, [i64, i64, P64]),
            "orc_rand_perm_exstack": (C.c_int, [i64, i64, i64, P64]),
            "orc_write_dataset": (C.c_int, [C.c_char_p, P64, P64, i64, i64]),
            "orc_read_mm": (C.c_int, [C.c_char_p, P64, P64, P64]),
            "orc_num_cpus": (C.c_int, []),
            "orc_triangle_agi_alg1": (i64, [P64, P64, i64, P64, P64, i64, P64]),
            "orc_gen_uniform": (None, [P64, i64, i64, C.c_uint64, C.c_int]),
            "orc_gen_values": (None, [P64, i64, C.c_uint64, C.c_int]),
            "orc_histo_exstack_buffered": (C.c_int, [P64, i64, P64, i64]),
            "orc_ig_exstack_buffered": (C.c_int, [P64, P64, i64, P64, i64]),
            "orc_triangle_exstack_push_buffered": (i64, [P64, P64, i64, i64, i64, i64, P64]),
            "orc_triangle_agi_sampled": (i64, [P64, P64, i64, i64, i64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        self.lib = lib

    # seeded inputs (the reference arm's own, so it never loads the GPU library)
    def gen_uniform(self, n: int, rng: int, seed: int, nthreads: int = 0) -> np.ndarray:
        out = np.empty(n, np.int64)
        self.lib.orc_gen_uniform(_p(out), n, rng, seed, nthreads)
        return out

    def gen_values(self, n: int, seed: int, nthreads: int = 0) -> np.ndarray:
        out = np.empty(n, np.int64)
        self.lib.orc_gen_values(_p(out), n, seed, nthreads)
        return out

    # histo -----------------------------------------------------------------
    def histo_agi(self, index: np.ndarray, counts: np.ndarray) -> None:
        self.lib.orc_histo_agi(_p(index), index.size, _p(counts))

    def histo_exstack(self, pckindx: np.ndarray, counts: np.ndarray) -> None:
        self.lib.orc_histo_exstack(_p(pckindx), pckindx.size, _p(counts))

    def histo_exstack_buffered(self, pckindx: np.ndarray, counts: np.ndarray, buf_cnt: int = 1024) -> None:
        """histo_exstack at one PE through buf_cnt-package exstack buffers."""
        if self.lib.orc_histo_exstack_buffered(_p(pckindx), pckindx.size, _p(counts), buf_cnt) != 0:
            raise ValueError("histo_exstack_buffered: bad buffer size")

    def histo_agi_mt(self, index: np.ndarray, counts: np.ndarray, nthreads: int = 0) -> None:
        self.lib.orc_histo_agi_mt(_p(index), index.size, _p(counts), nthreads)

    # ig --------------------------------------------------------------------
    def ig_agi(self, index: np.ndarray, table: np.ndarray) -> np.ndarray:
        tgt = np.empty(index.size, np.int64)
        self.lib.orc_ig_agi(_p(tgt), _p(index), index.size, _p(table))
        return tgt

    def ig_exstack(self, pckindx: np.ndarray, table: np.ndarray) -> np.ndarray:
        tgt = np.empty(pckindx.size, np.int64)
        self.lib.orc_ig_exstack(_p(tgt), _p(pckindx), pckindx.size, _p(table))
        return tgt

    def ig_exstack_buffered(self, pckindx: np.ndarray, table: np.ndarray, buf_cnt: int = 1024) -> np.ndarray:
        """ig_exstack at one PE through buf_cnt-package exstack buffers."""
        tgt = np.empty(pckindx.size, np.int64)
        if self.lib.orc_ig_exstack_buffered(_p(tgt), _p(pckindx), pckindx.size, _p(table), buf_cnt) != 0:
            raise ValueError("ig_exstack_buffered: bad buffer size")
        return tgt

    def ig_agi_mt(self, tgt: np.ndarray, index: np.ndarray, table: np.ndarray, nthreads: int = 0) -> None:
        self.lib.orc_ig_agi_mt(_p(tgt), _p(index), index.size, _p(table), nthreads)

    # triangles ---------------------------------------------------------------
    def triangle_agi(self, offset: np.ndarray, nonzero: np.ndarray) -> tuple[int, int]:
        pulled = C.c_int64(0)
        c = self.lib.orc_triangle_agi(_p(offset), _p(nonzero), offset.size - 1, C.byref(pulled))
        return int(c), int(pulled.value)

    def triangle_agi_alg1(self, loff: np.ndarray, lcol: np.ndarray, uoff: np.ndarray,
                          ucol: np.ndarray) -> tuple[int, int]:
        """alg 1: sum over L's nonzeros (i,j) of |U_i and U_j| and the tally."""
        pulled = C.c_int64(0)
        c = self.lib.orc_triangle_agi_alg1(_p(loff), _p(lcol), loff.size - 1, _p(uoff), _p(ucol), ucol.size,
                                           C.byref(pulled))
        return int(c), int(pulled.value)

    def triangle_exstack_push(self, offset: np.ndarray, nonzero: np.ndarray) -> tuple[int, int]:
        pushed = C.c_int64(0)
        c = self.lib.orc_triangle_exstack_push(_p(offset), _p(nonzero), offset.size - 1, C.byref(pushed))
        return int(c), int(pushed.value)

    def triangle_exstack_push_buffered(self, offset: np.ndarray, nonzero: np.ndarray, bufsiz: int = 1024,
                                       row0: int = 0, row_step: int = 1) -> tuple[int, int]:
        """triangle_exstack_push (alg 0) at one PE through bufsiz-package
        buffers, over rows row0, row0 + row_step, ..."""
        pushed = C.c_int64(0)
        c = self.lib.orc_triangle_exstack_push_buffered(_p(offset), _p(nonzero), offset.size - 1, bufsiz, row0,
                                                        row_step, C.byref(pushed))
        if c < 0:
            raise ValueError("triangle_exstack_push_buffered: bad arguments")
        return int(c), int(pushed.value)

    def triangle_agi_sampled(self, offset: np.ndarray, nonzero: np.ndarray, row0: int, row_step: int) -> int:
        """The AGI loop (alg 0) over rows row0, row0 + row_step, ..."""
        return int(self.lib.orc_triangle_agi_sampled(_p(offset), _p(nonzero), offset.size - 1, row0, row_step))

    def triangle_work(self, offset: np.ndarray, nonzero: np.ndarray) -> tuple[int, int]:
        pl, ps = C.c_int64(0), C.c_int64(0)
        self.lib.orc_triangle_work(_p(offset), _p(nonzero), offset.size - 1, C.byref(pl), C.byref(ps))
        return int(pl.value), int(ps.value)

    def is_strict_lower_tidy(self, offset: np.ndarray, nonzero: np.ndarray) -> bool:
        return bool(self.lib.orc_is_strict_lower_tidy(_p(offset), _p(nonzero), offset.size - 1))

    def triangle_agi_mt(self, offset: np.ndarray, nonzero: np.ndarray, nthreads: int = 0) -> int:
        return int(self.lib.orc_triangle_agi_mt(_p(offset), _p(nonzero), offset.size - 1, nthreads))

    def transpose(self, offset: np.ndarray, nonzero: np.ndarray, numcols: int) -> tuple[np.ndarray, np.ndarray]:
        toff = np.zeros(numcols + 1, np.int64)
        tcol = np.zeros(max(nonzero.size, 1), np.int64)
        if self.lib.orc_transpose(_p(offset), _p(nonzero), offset.size - 1, numcols, _p(toff), _p(tcol)) != 0:
            raise ValueError("column outside [0, numcols)")
        return toff, tcol[: nonzero.size]

    def permute(self, offset: np.ndarray, nonzero: np.ndarray, rperminv: np.ndarray,
                cperminv: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        poff = np.zeros(offset.size, np.int64)
        pcol = np.zeros(max(nonzero.size, 1), np.int64)
        self.lib.orc_permute(_p(offset), _p(nonzero), offset.size - 1, _p(rperminv), _p(cperminv), _p(poff), _p(pcol))
        return poff, pcol[: nonzero.size]

    def rand_perm(self, n: int, seed: int) -> np.ndarray:
        out = np.zeros(max(n, 1), np.int64)
        if self.lib.orc_rand_perm(n, seed, _p(out)) != 0:
            raise MemoryError("orc_rand_perm")
        return out[:n]

    def rand_perm_exstack(self, n: int, seed: int, buf_cnt: int = 1024) -> np.ndarray:
        out = np.zeros(max(n, 1), np.int64)
        if self.lib.orc_rand_perm_exstack(n, seed, buf_cnt, _p(out)) != 0:
            raise MemoryError("orc_rand_perm_exstack")
        return out[:n]

    def write_dataset(self, offset: np.ndarray, nonzero: np.ndarray, numcols: int, dirname) -> None:
        if self.lib.orc_write_dataset(str(dirname).encode(), _p(offset), _p(nonzero), offset.size - 1,
                                      numcols) != 0:
            raise OSError(f"orc_write_dataset: {dirname}")

    def read_mm(self, path) -> tuple[np.ndarray, np.ndarray, int]:
        dims = np.zeros(3, np.int64)
        if self.lib.orc_read_mm(str(path).encode(), _p(dims), None, None) != 0:
            raise ValueError(f"{path}: rejected")
        nr, nc, nnz = (int(x) for x in dims)
        off = np.zeros(nr + 1, np.int64)
        col = np.zeros(max(nnz, 1), np.int64)
        if self.lib.orc_read_mm(str(path).encode(), _p(dims), _p(off), _p(col)) != 0:
            raise ValueError(f"{path}: rejected")
        return off, col[:nnz], nc

    def num_cpus(self) -> int:
        return int(self.lib.orc_num_cpus())


class _sparsemat_t(C.Structure):
    _fields_ = [(n, i64) for n in ("local", "numrows", "lnumrows", "numcols", "nnz", "lnnz")] + [
        (n, P64) for n in ("offset", "loffset", "nonzero", "lnonzero")]


class Reference:
    """The reference's own functions (oracle/_ref/libbale_ref.so), one PE."""

    def __init__(self, path: Path | None = None):
        path = path or REF_LIB
        if not path.exists():
            raise FileNotFoundError(f"{path} is not built (needs the reference tree)")
        lib = C.CDLL(str(path))
        PS = C.POINTER(_sparsemat_t)
        sig = {
            "histo_agi": (C.c_double, [P64, i64, P64]),
            "histo_exstack": (C.c_double, [P64, i64, P64, i64]),
            "histo_exstack2": (C.c_double, [P64, i64, P64, i64]),
            "ig_agi": (C.c_double, [P64, P64, i64, P64]),
            "ig_exstack": (C.c_double, [P64, P64, i64, P64, i64]),
            "ig_exstack2": (C.c_double, [P64, P64, i64, P64, i64]),
            "triangle_agi": (C.c_double, [P64, P64, PS, PS, i64]),
            "triangle_exstack_push": (C.c_double, [P64, P64, PS, PS, i64, i64]),
            "triangle_exstack2_push": (C.c_double, [P64, P64, PS, PS, i64, i64]),
            "triangle_agi_iter": (C.c_double, [P64, P64, PS, PS, i64]),
            "gen_erdos_renyi_graph_dist": (PS, [C.c_int, C.c_double, i64, i64, i64]),
            "gen_local_mat_from_stars": (PS, [i64, P64, C.c_int]),
            "kron_prod_dist": (PS, [PS, PS, i64]),
            "clear_matrix": (None, [PS]),
            "transpose_matrix_agi": (PS, [PS]),
            "permute_matrix_agi": (PS, [PS, P64, P64]),
            "rand_permp_agi": (P64, [i64, C.c_int]),
            "rand_permp_exstack": (P64, [i64, C.c_int, i64]),
            "rand_permp": (P64, [i64, C.c_int]),
            "rand_permp_exstack2": (P64, [i64, C.c_int, i64]),
            "write_matrix_mm": (C.c_int, [PS, C.c_char_p]),
            "read_matrix_mm_to_dist": (PS, [C.c_char_p]),
            "write_sparse_matrix_agi": (i64, [C.c_char_p, PS]),
            "write_sparse_matrix_exstack": (i64, [C.c_char_p, PS, i64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        self.lib = lib
        self._PS = PS

    def _mat(self, offset: np.ndarray, nonzero: np.ndarray):
        n = offset.size - 1
        po, pn = _p(offset), _p(nonzero)
        return _sparsemat_t(0, n, n, n, nonzero.size, nonzero.size, po, po, pn, pn)

    def triangles(self, offset: np.ndarray, nonzero: np.ndarray) -> dict[str, tuple[int, int]]:
        """count and shared-refs/pushes of every variant the oracle build has."""
        m = self._mat(offset, nonzero)
        out = {}
        for name, extra in (("triangle_agi", ()), ("triangle_exstack_push", (1024,)),
                            ("triangle_exstack2_push", (1024,)), ("triangle_agi_iter", ())):
            cnt, sr = C.c_int64(0), C.c_int64(0)
            t = getattr(self.lib, name)(C.byref(cnt), C.byref(sr), C.byref(m), None, 0, *extra)
            if t < 0:
                raise RuntimeError(f"reference {name} failed")
            out[name] = (int(cnt.value), int(sr.value))
        return out

    def _unpack(self, m) -> tuple[np.ndarray, np.ndarray]:
        s = m.contents
        off = np.ctypeslib.as_array(s.loffset, shape=(s.lnumrows + 1,)).copy()
        col = np.ctypeslib.as_array(s.lnonzero, shape=(s.lnnz,)).copy() if s.lnnz else np.zeros(0, np.int64)
        self.lib.clear_matrix(m)
        return off, col

    def transpose(self, offset: np.ndarray, nonzero: np.ndarray, numcols: int) -> tuple[np.ndarray, np.ndarray]:
        """spmat's transpose_matrix_agi (spmat/spmat_agi.upc:180-235) at one PE."""
        n = offset.size - 1
        po, pn = _p(offset), _p(nonzero)
        m = _sparsemat_t(0, n, n, numcols, nonzero.size, nonzero.size, po, po, pn, pn)
        return self._unpack(self.lib.transpose_matrix_agi(C.byref(m)))

    def permute(self, offset: np.ndarray, nonzero: np.ndarray, numcols: int, rperminv: np.ndarray,
                cperminv: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """spmat's permute_matrix_agi (spmat/spmat_agi.upc:119-173) at one PE."""
        n = offset.size - 1
        po, pn = _p(offset), _p(nonzero)
        m = _sparsemat_t(0, n, n, numcols, nonzero.size, nonzero.size, po, po, pn, pn)
        return self._unpack(self.lib.permute_matrix_agi(C.byref(m), _p(rperminv), _p(cperminv)))

    def write_mm(self, offset: np.ndarray, nonzero: np.ndarray, numcols: int, path: str) -> None:
        """spmat's write_matrix_mm (spmat/spmat_utils.upc:128-149) at one PE."""
        n = offset.size - 1
        po, pn = _p(offset), _p(nonzero)
        m = _sparsemat_t(0, n, n, numcols, nonzero.size, nonzero.size, po, po, pn, pn)
        if self.lib.write_matrix_mm(C.byref(m), path.encode()) != 0:
            raise RuntimeError("write_matrix_mm failed")

    def write_dataset(self, offset: np.ndarray, nonzero: np.ndarray, numcols: int, dirname: str,
                      buf_cnt: int | None = None) -> None:
        """spmat's write_sparse_matrix_agi (spmat/spmat_agi.upc:286-335), or
        with buf_cnt write_sparse_matrix_exstack (spmat/spmat_exstack.upc:
        494-686), at one PE.  Its file names live in 64-byte buffers: keep
        dirname short."""
        n = offset.size - 1
        po, pn = _p(offset), _p(nonzero)
        m = _sparsemat_t(0, n, n, numcols, nonzero.size, nonzero.size, po, po, pn, pn)
        if len(dirname) > 40:
            raise ValueError("dirname too long for the reference's 64-byte file names")
        if buf_cnt is None:
            rc = self.lib.write_sparse_matrix_agi(dirname.encode(), C.byref(m))
        else:
            rc = self.lib.write_sparse_matrix_exstack(dirname.encode(), C.byref(m), buf_cnt)
            # it leaves rowcnt_0 and nonzero_0 open (no fclose): the bytes sit
            # in stdio buffers until exit, so flush every open stream
            C.CDLL(None).fflush(None)
        if rc != 0:
            raise RuntimeError("write_sparse_matrix failed")

    def read_mm(self, path: str) -> tuple[np.ndarray, np.ndarray, int]:
        """spmat's read_matrix_mm_to_dist (spmat/spmat_utils.upc:217-370) at one PE."""
        m = self.lib.read_matrix_mm_to_dist(path.encode())
        if not m:
            raise RuntimeError("read_matrix_mm_to_dist failed")
        nc = m.contents.numcols
        off, col = self._unpack(m)
        return off, col, nc

    def rand_perm(self, n: int, seed: int) -> np.ndarray:
        """spmat's rand_permp_agi (spmat/spmat_agi.upc:56-107) at one PE: darts
        from lrand48 after srand48(seed) (seed != 0)."""
        p = self.lib.rand_permp_agi(n, seed)
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    def rand_perm_exstack(self, n: int, seed: int, buf_cnt: int = 1024) -> np.ndarray:
        """spmat's rand_permp_exstack (spmat/spmat_exstack.upc:62-190) at one
        PE; rand_permp (spmat/spmat_utils.upc:63-74) calls it with 1024."""
        p = self.lib.rand_permp_exstack(n, seed, buf_cnt)
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    def rand_perm_exstack2(self, n: int, seed: int, buf_cnt: int = 1024) -> np.ndarray:
        """spmat's rand_permp_exstack2 (spmat/spmat_exstack2.upc:60-73) at one PE."""
        p = self.lib.rand_permp_exstack2(n, seed, buf_cnt)
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    def rand_permp(self, n: int, seed: int) -> np.ndarray:
        """spmat's rand_permp (spmat/spmat_utils.upc:63-74) at one PE."""
        p = self.lib.rand_permp(n, seed)
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    def kronecker_lower(self, mode: int, specs) -> tuple[np.ndarray, np.ndarray]:
        """The triangle app's -K graph (apps/triangle_src/triangle.upc:147-168,
        :297-299): the specs split in half, each half a local product of stars
        (gen_local_mat_from_stars), combined by kron_prod_dist(B, C, lower=1)
        (spmat/spmat_utils.upc:813-1049), at one PE."""
        sp = np.ascontiguousarray(np.asarray(specs, dtype=np.int64))
        half = sp.size // 2
        b_spec, c_spec = np.ascontiguousarray(sp[:half]), np.ascontiguousarray(sp[half:])
        B = self.lib.gen_local_mat_from_stars(b_spec.size, _p(b_spec), mode)
        Cm = self.lib.gen_local_mat_from_stars(c_spec.size, _p(c_spec), mode)
        if not B or not Cm:
            raise RuntimeError("gen_local_mat_from_stars failed")
        A = self.lib.kron_prod_dist(B, Cm, 1)
        self.lib.clear_matrix(B)
        self.lib.clear_matrix(Cm)
        if not A:
            raise RuntimeError("kron_prod_dist failed")
        return self._unpack(A)

    def erdos_renyi_lower(self, n: int, p: float, seed: int) -> tuple[np.ndarray, np.ndarray]:
        """spmat's gen_erdos_renyi_graph_dist(n, p, 0, mode 1 = lower, seed)
        (spmat/spmat_utils.upc:554-573) at one PE."""
        m = self.lib.gen_erdos_renyi_graph_dist(n, p, 0, 1, seed)
        s = m.contents
        off = np.ctypeslib.as_array(s.loffset, shape=(s.lnumrows + 1,)).copy()
        col = np.ctypeslib.as_array(s.lnonzero, shape=(s.lnnz,)).copy() if s.lnnz else np.zeros(0, np.int64)
        self.lib.clear_matrix(m)
        return off, col
