"""ctypes access to the CPU checkers (test infrastructure only).

* ``cluster``      -> oracle/_build/libhpdoracle.so, the C restatement (hpd_oracle.c)
* ``ref_cluster``  -> oracle/_ref/libhpdref.so, the upstream headers compiled unmodified
                      with the upstream flags on this host (from the upstream checkout,
                      or from the copy `make -C oracle stage` leaves in oracle/_ref/upstream)

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libhpdoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libhpdref.so")
REF_ROOT = os.environ.get("HPD_REF_ROOT", "/root/reference")
REF_INCLUDE = os.path.join(REF_ROOT, "include")
# the upstream headers staged unmodified by `make -C oracle stage` (git-ignored), so
# that a host without the upstream checkout can build the reference from them
REF_STAGED = os.path.join(HERE, "_ref", "upstream", "include")

CELL_RECIP, CELL_DIV = 0, 1
DIST_GCC_X86, DIST_SEQ, DIST_SEQ_FMA, DIST_GCC_AARCH64 = 0, 1, 2, 3

DTYPES = {
    np.dtype(np.float32): 0, np.dtype(np.float64): 1,
    np.dtype(np.int8): 2, np.dtype(np.int16): 3, np.dtype(np.int32): 4, np.dtype(np.int64): 5,
    np.dtype(np.uint8): 6, np.dtype(np.uint16): 7, np.dtype(np.uint32): 8, np.dtype(np.uint64): 9,
}

_lib = None
_ref = None


def ref_sources_available() -> bool:
    return os.path.exists(os.path.join(REF_INCLUDE, "hpdbscan.h")) or \
        os.path.exists(os.path.join(REF_STAGED, "hpdbscan.h"))


def build(ref: bool | None = None) -> None:
    """Compile the restatement (always) and the upstream build (when its sources exist:
    the upstream checkout, which is then also staged, or a staged copy)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref is None:
        ref = ref_sources_available()
    if ref:
        if os.path.exists(os.path.join(REF_INCLUDE, "hpdbscan.h")):
            subprocess.run(["make", "-s", "-C", HERE, "stage", f"REF_ROOT={REF_ROOT}"], check=True)
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={REF_ROOT}"], check=True)


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        lib = ctypes.CDLL(ORACLE_SO)
        lib.hpd_oracle_cluster.restype = ctypes.c_int
        lib.hpd_oracle_cluster.argtypes = [
            ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
            ctypes.c_uint64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.hpd_oracle_last_error.restype = ctypes.c_char_p
        _lib = lib
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def _load_ref():
    global _ref
    if _ref is None:
        lib = ctypes.CDLL(REF_SO)
        lib.hpdref_cluster.restype = ctypes.c_int
        lib.hpdref_cluster.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_float, ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p]
        lib.hpdref_index.restype = ctypes.c_int
        lib.hpdref_index.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.hpdref_last_error.restype = ctypes.c_char_p
        lib.hpdref_max_threads.restype = ctypes.c_int
        _ref = lib
    return _ref


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


def cluster(points, eps, min_points, threads=1, cell_mode=CELL_RECIP, dist_mode=DIST_GCC_X86,
            with_order=False):
    """Labels in input order (int64), optionally with the sorted order and cell ids."""
    pts = np.ascontiguousarray(points)
    n, d = pts.shape
    lib = _load()
    labels = np.empty(n, np.int64)
    order = np.empty(n, np.int64) if with_order else None
    cells = np.empty(n, np.uint64) if with_order else None
    rc = lib.hpd_oracle_cluster(
        pts.ctypes.data, n, d, DTYPES[pts.dtype], ctypes.c_float(eps), min_points, threads,
        cell_mode, dist_mode, labels.ctypes.data,
        order.ctypes.data if with_order else None, cells.ctypes.data if with_order else None)
    if rc:
        raise OracleError(rc, lib.hpd_oracle_last_error().decode())
    return (labels, order, cells) if with_order else labels


def ref_cluster(points, eps, min_points, threads=1):
    pts = np.ascontiguousarray(points)
    n, d = pts.shape
    lib = _load_ref()
    out = np.empty(n, np.int64)
    rc = lib.hpdref_cluster(pts.ctypes.data, n, d, DTYPES[pts.dtype], ctypes.c_float(eps),
                            min_points, threads, out.ctypes.data)
    if rc:
        raise OracleError(rc, lib.hpdref_last_error().decode())
    return out


def ref_index(points, eps):
    """Upstream SpatialIndex: (cell id, original index) in sorted order, cells/dim, dim order."""
    pts = np.ascontiguousarray(points)
    n, d = pts.shape
    lib = _load_ref()
    cells = np.empty(n, np.int64)
    order = np.empty(n, np.int64)
    dims = np.empty(2 * d, np.int64)
    rc = lib.hpdref_index(pts.ctypes.data, n, d, DTYPES[pts.dtype], ctypes.c_float(eps),
                          cells.ctypes.data, order.ctypes.data, dims.ctypes.data)
    if rc:
        raise OracleError(rc, lib.hpdref_last_error().decode())
    return cells.astype(np.uint64), order, dims[:d], dims[d:]
