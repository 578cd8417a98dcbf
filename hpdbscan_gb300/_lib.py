"""ctypes binding of libhpdbscan_gb300.so (the C ABI in include/hpdbscan_gb300.h).

The library is built in-tree by ``hpdbscan_gb300.build``; when it is missing this
module raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

HPD_OK, HPD_ERR_INVALID, HPD_ERR_UNSUPPORTED, HPD_ERR_RUNTIME = 0, 1, 2, 3
HPD_ERR_GRID, HPD_ERR_NOMEM, HPD_ERR_CUDA, HPD_ERR_TIMEOUT = 4, 5, 6, 7

F32, F64, I8, I16, I32, I64, U8, U16, U32, U64 = range(10)
CELL_RECIP, CELL_DIV = 0, 1
DIST_GCC_X86, DIST_SEQ, DIST_SEQ_FMA, DIST_GCC_AARCH64 = 0, 1, 2, 3
TIE_EXACT, TIE_SMALLEST_ID = 0, 1
DIAG_COUNT_PAIRS = 1
INJECT_FAIL_ALLOC = 1

EXPORTS = ("hpd_create", "hpd_destroy", "hpd_set_arith", "hpd_set_tie_break", "hpd_set_tie_pass_limit",
           "hpd_set_tuning", "hpd_set_tuning_table",
           "hpd_set_diagnostics", "hpd_debug_inject", "hpd_cluster", "hpd_cluster_device",
           "hpd_get_stats", "hpd_last_error", "hpd_version", "hpd_cluster_device_noalloc",
           "hpd_noalloc_last_error", "hpd_cluster_batch", "hpd_server_create", "hpd_server_submit",
           "hpd_server_poll", "hpd_server_wait", "hpd_server_destroy", "hpd_server_last_error",
           "hpd_h5_read", "hpd_h5_free", "hpd_h5_write")


class Job(ctypes.Structure):
    """hpd_job of include/hpdbscan_gb300.h."""
    _fields_ = [("data", ctypes.c_void_p), ("n", ctypes.c_int64), ("d", ctypes.c_int32), ("dtype", ctypes.c_int32),
                ("epsilon", ctypes.c_float), ("min_points", ctypes.c_uint64), ("cell_mode", ctypes.c_int32),
                ("dist_mode", ctypes.c_int32), ("labels", ctypes.c_void_p), ("status", ctypes.c_int32),
                ("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double), ("deadline_ms", ctypes.c_double)]


class Tuning(ctypes.Structure):
    """hpd_tuning of include/hpdbscan_gb300.h (0: built-in default)."""
    _fields_ = [("sparse_queries", ctypes.c_int32), ("dense_min_points", ctypes.c_int32),
                ("greedy_tiles", ctypes.c_int32)]


class TuningEntry(ctypes.Structure):
    _fields_ = [("max_points", ctypes.c_int64), ("dims", ctypes.c_int32), ("tuning", Tuning)]


class Stats(ctypes.Structure):
    _fields_ = [("total_ms", ctypes.c_double), ("index_ms", ctypes.c_double), ("core_ms", ctypes.c_double),
                ("union_ms", ctypes.c_double), ("border_ms", ctypes.c_double), ("tie_ms", ctypes.c_double),
                ("finalize_ms", ctypes.c_double),
                ("n_cells", ctypes.c_int64), ("n_core", ctypes.c_int64), ("n_ambiguous", ctypes.c_int64),
                ("tie_iterations", ctypes.c_int64), ("kernel_launches", ctypes.c_int64),
                ("extent_ms", ctypes.c_double), ("cells_sort_ms", ctypes.c_double), ("cell_table_ms", ctypes.c_double),
                ("cell_ids_ms", ctypes.c_double), ("rules_ms", ctypes.c_double), ("core_pairs", ctypes.c_int64)]


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load the engine library.  Raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run `python -m hpdbscan_gb300.build` first")
        _build.build()
    lib = ctypes.CDLL(path)
    H = ctypes.c_void_p
    lib.hpd_create.argtypes = [ctypes.c_float, ctypes.c_uint64, ctypes.POINTER(H)]
    lib.hpd_create.restype = ctypes.c_int
    lib.hpd_destroy.argtypes = [H]
    lib.hpd_destroy.restype = None
    lib.hpd_set_arith.argtypes = [H, ctypes.c_int, ctypes.c_int]
    lib.hpd_set_arith.restype = ctypes.c_int
    lib.hpd_set_tie_break.argtypes = [H, ctypes.c_int]
    lib.hpd_set_tie_break.restype = ctypes.c_int
    for name in ("hpd_set_tie_pass_limit", "hpd_set_diagnostics", "hpd_debug_inject"):
        getattr(lib, name).argtypes = [H, ctypes.c_int32]
        getattr(lib, name).restype = ctypes.c_int
    lib.hpd_set_tuning.argtypes = [H, ctypes.POINTER(Tuning)]
    lib.hpd_set_tuning.restype = ctypes.c_int
    lib.hpd_set_tuning_table.argtypes = [ctypes.POINTER(TuningEntry), ctypes.c_int32]
    lib.hpd_set_tuning_table.restype = ctypes.c_int
    lib.hpd_cluster.argtypes = [H, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                ctypes.c_void_p]
    lib.hpd_cluster.restype = ctypes.c_int
    lib.hpd_cluster_device.argtypes = [H, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                       ctypes.c_void_p, ctypes.c_void_p]
    lib.hpd_cluster_device.restype = ctypes.c_int
    lib.hpd_get_stats.argtypes = [H, ctypes.POINTER(Stats)]
    lib.hpd_get_stats.restype = ctypes.c_int
    lib.hpd_last_error.argtypes = []
    lib.hpd_last_error.restype = ctypes.c_char_p
    lib.hpd_version.argtypes = []
    lib.hpd_version.restype = ctypes.c_char_p
    lib.hpd_cluster_device_noalloc.argtypes = [ctypes.c_float, ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32,
                                               ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                               ctypes.c_void_p, ctypes.c_void_p]
    lib.hpd_cluster_device_noalloc.restype = ctypes.c_int
    lib.hpd_noalloc_last_error.argtypes = []
    lib.hpd_noalloc_last_error.restype = ctypes.c_char_p
    lib.hpd_cluster_batch.argtypes = [ctypes.POINTER(Job), ctypes.c_int64, ctypes.c_int32]
    lib.hpd_cluster_batch.restype = ctypes.c_int
    lib.hpd_server_create.argtypes = [ctypes.c_int32, ctypes.c_uint64, ctypes.c_int64, ctypes.c_int32,
                                      ctypes.POINTER(H)]
    lib.hpd_server_create.restype = ctypes.c_int
    lib.hpd_server_submit.argtypes = [H, ctypes.POINTER(Job), ctypes.POINTER(ctypes.c_int64)]
    lib.hpd_server_submit.restype = ctypes.c_int
    lib.hpd_server_poll.argtypes = [H, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32)]
    lib.hpd_server_poll.restype = ctypes.c_int
    lib.hpd_server_wait.argtypes = [H, ctypes.c_int64]
    lib.hpd_server_wait.restype = ctypes.c_int
    lib.hpd_server_destroy.argtypes = [H]
    lib.hpd_server_destroy.restype = None
    lib.hpd_server_last_error.argtypes = []
    lib.hpd_server_last_error.restype = ctypes.c_char_p
    lib.hpd_h5_read.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p),
                                ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32),
                                ctypes.POINTER(ctypes.c_int32)]
    lib.hpd_h5_read.restype = ctypes.c_int
    lib.hpd_h5_free.argtypes = [ctypes.c_void_p]
    lib.hpd_h5_free.restype = None
    lib.hpd_h5_write.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64]
    lib.hpd_h5_write.restype = ctypes.c_int
    _lib = lib
    return lib


def raise_for(code: int) -> None:
    """Map a status code to the exception the upstream SWIG module raises."""
    if code == HPD_OK:
        return
    msg = load().hpd_last_error().decode(errors="replace")
    if code in (HPD_ERR_INVALID, HPD_ERR_UNSUPPORTED):
        raise ValueError(msg)
    if code == HPD_ERR_NOMEM:
        raise MemoryError(msg)
    raise RuntimeError(msg)
