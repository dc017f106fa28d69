"""ctypes binding of libbale_gb300.so (the C ABI in include/bale_gb300.h and
include/bale_inputs.h).  Importing this module never falls back to anything:
if the shared library is missing it raises, naming the build command."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libbale_gb300.so"

i64 = C.c_int64
u64 = C.c_uint64
P64 = C.POINTER(C.c_int64)
VP = C.c_void_p


class sparsemat_t(C.Structure):
    """Layout of the reference's sparsemat_t (spmat/spmat.h:73-86)."""

    _fields_ = [
        ("local", i64), ("numrows", i64), ("lnumrows", i64), ("numcols", i64),
        ("nnz", i64), ("lnnz", i64),
        ("offset", P64), ("loffset", P64), ("nonzero", P64), ("lnonzero", P64),
    ]


PSM = C.POINTER(sparsemat_t)


class bale_instance_t(C.Structure):
    """One instance of a batch (include/bale_gb300.h)."""

    _fields_ = [("kind", C.c_int32), ("shift", C.c_int32), ("n", i64), ("m", i64),
                ("out", VP), ("inp", VP), ("aux", VP)]


PINST = C.POINTER(bale_instance_t)


class bale_request_t(C.Structure):
    """One request of a serving trace (include/bale_gb300.h)."""

    _fields_ = [("kind", C.c_int32), ("object", C.c_int32), ("shift", C.c_int32), ("reserved", C.c_int32),
                ("n", i64), ("index", VP), ("out", VP), ("arrival", C.c_double)]


class bale_serve_stats_t(C.Structure):
    _fields_ = [(f, C.c_double) for f in ("makespan_s", "p50_s", "p99_s", "mean_s", "items_per_s", "gpu_busy_s")] + \
               [(f, i64) for f in ("ticks", "tasks", "max_active", "admission_waits", "bad", "loop_iters", "express")]

# name -> (restype, argtypes)
SIGNATURES: dict[str, tuple[object, list[object]]] = {
    # drop-ins (apps/histo_src/histo.h:47-50)
    "histo_agi": (C.c_double, [P64, i64, P64]),
    "histo_exstack": (C.c_double, [P64, i64, P64, i64]),
    "histo_exstack2": (C.c_double, [P64, i64, P64, i64]),
    "histo_conveyor": (C.c_double, [P64, i64, P64]),
    # apps/ig_src/ig.h:49-52
    "ig_agi": (C.c_double, [P64, P64, i64, P64]),
    "ig_exstack": (C.c_double, [P64, P64, i64, P64, i64]),
    "ig_exstack2": (C.c_double, [P64, P64, i64, P64, i64]),
    "ig_conveyor": (C.c_double, [P64, P64, i64, P64]),
    # apps/triangle_src/triangle.h:50-61
    "triangle_agi": (C.c_double, [P64, P64, PSM, PSM, i64]),
    "triangle_exstack_push": (C.c_double, [P64, P64, PSM, PSM, i64, i64]),
    "triangle_exstack2_push": (C.c_double, [P64, P64, PSM, PSM, i64, i64]),
    "triangle_convey_push": (C.c_double, [P64, P64, PSM, PSM, i64]),
    "triangle_agi_iter": (C.c_double, [P64, P64, PSM, PSM, i64]),
    # library state
    "bale_last_error": (C.c_char_p, []),
    "bale_version": (C.c_char_p, []),
    "bale_device_caps": (C.c_int, [P64, C.c_int]),
    "bale_release_buffers": (None, []),
    # tuning knobs
    "bale_tune_set": (C.c_int, [C.c_char_p, i64]),
    "bale_tune_get": (i64, [C.c_char_p]),
    "bale_tune_count": (C.c_int, []),
    "bale_tune_load": (C.c_int, [C.c_char_p]),
    "bale_tune_name": (C.c_char_p, [C.c_int]),
    # device-resident
    "bale_histo_dev": (C.c_int, [VP, i64, VP, i64, C.c_int, VP, VP]),
    "bale_ig_dev": (C.c_int, [VP, VP, i64, VP, i64, C.c_int, VP, VP]),
    "bale_triangle_dev": (C.c_int, [VP, VP, i64, i64, VP, VP, VP, VP]),
    "bale_l2_red_rate": (C.c_int, [VP, i64, i64, VP]),
    "bale_graph_build_dev": (C.c_int, [VP, VP, i64, i64, VP, VP, P64, VP]),
    "bale_graph_build_workspace": (i64, [i64, i64]),
    "bale_gen_rmat_dev": (C.c_int, [i64, i64, C.c_double, C.c_double, C.c_double, C.c_uint64, VP, VP, P64, VP]),
    "bale_transpose_dev": (C.c_int, [VP, VP, i64, i64, i64, VP, VP, VP]),
    "bale_permute_dev": (C.c_int, [VP, VP, i64, i64, i64, VP, VP, VP, VP, VP]),
    "bale_rand_perm_dev": (C.c_int, [i64, C.c_uint64, VP, VP]),
    "bale_rand_perm_exstack_dev": (C.c_int, [i64, C.c_uint64, i64, VP, VP]),
    "bale_rand_perm_exstack2_dev": (C.c_int, [i64, C.c_uint64, i64, VP, VP]),
    "bale_write_matrix_mm": (C.c_int, [C.POINTER(sparsemat_t), C.c_char_p]),
    "bale_mm_header": (C.c_int, [C.c_char_p, P64, P64, P64, P64, C.POINTER(C.c_int)]),
    "bale_read_matrix_mm_dev": (C.c_int, [C.c_char_p, VP, VP, VP]),
    "bale_write_sparse_matrix": (C.c_int, [C.c_char_p, C.POINTER(sparsemat_t)]),
    "bale_write_sparse_matrix_dev": (C.c_int, [C.c_char_p, VP, VP, i64, i64, i64, i64, VP]),
    "bale_sparse_matrix_header": (C.c_int, [C.c_char_p, P64, P64, P64, P64]),
    "bale_read_sparse_matrix_dev": (C.c_int, [C.c_char_p, VP, VP, VP]),
    "bale_triangle_prepare": (VP, [VP, VP, i64, i64, VP, VP]),
    "bale_triangle_count_prepared": (C.c_int, [VP, VP, VP, VP]),
    "bale_triangle_release": (None, [VP]),
    "bale_batch_create": (VP, [PINST, i64]),
    "bale_batch_run": (C.c_int, [VP, VP]),
    "bale_batch_bad": (C.c_int, [VP, P64, i64]),
    "bale_batch_stats": (C.c_int, [VP, P64, C.c_int]),
    "bale_batch_plan": (C.c_int, [VP, P64, i64]),
    "bale_batch_destroy": (None, [VP]),
    "bale_server_create": (VP, [i64, C.c_int]),
    "bale_server_add_table": (C.c_int, [VP, P64, i64]),
    "bale_server_add_counts": (C.c_int, [VP, i64]),
    "bale_server_add_graph": (C.c_int, [VP, P64, P64, i64, i64]),
    "bale_server_read_counts": (C.c_int, [VP, C.c_int, P64, i64]),
    "bale_server_run": (C.c_int, [VP, C.POINTER(bale_request_t), i64, C.POINTER(C.c_double),
                                  C.POINTER(bale_serve_stats_t)]),
    "bale_server_destroy": (None, [VP]),
    "bale_ig_dev_noalloc": (C.c_int, [VP, VP, i64, VP, i64, C.c_int, VP, VP]),
    # inputs
    "bale_splitmix64": (u64, [u64, u64]),
    "bale_gen_uniform": (C.c_int, [P64, i64, i64, u64, C.c_int]),
    "bale_gen_values": (C.c_int, [P64, i64, u64]),
    "bale_gen_uniform_dev": (C.c_int, [VP, i64, i64, u64, C.c_int, VP]),
    "bale_gen_values_dev": (C.c_int, [VP, i64, u64, VP]),
    "bale_gen_negative_table": (C.c_int, [P64, i64]),
    "bale_gen_zipf": (C.c_int, [P64, i64, i64, C.c_double, u64, u64, C.c_int]),
    "bale_keyed_perm": (i64, [i64, i64, u64]),
    "bale_gen_rmat": (PSM, [i64, i64, C.c_double, C.c_double, C.c_double, u64]),
    "bale_gen_erdos_renyi": (PSM, [i64, C.c_double, u64]),
    "bale_gen_kronecker": (PSM, [C.c_int, P64, i64]),
    "bale_kronecker_triangles": (i64, [C.c_int, P64, i64]),
    "bale_make_matrix": (PSM, [i64, i64, i64]),
    "bale_free_matrix": (None, [PSM]),
    "bale_set_host_threads": (None, [C.c_int]),
}

_lib: C.CDLL | None = None


def load() -> C.CDLL:
    """Load libbale_gb300.so once and declare every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is not built; run `python bale_old_gb300/build.py` "
            "(or __graft_entry__.build())")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
