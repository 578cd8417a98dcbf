"""Python mirror of the upstream ``hpdbscan`` module (swig/hpdbscan.i).

    >>> from hpdbscan_gb300 import HPDBSCAN
    >>> labels = HPDBSCAN(epsilon=0.3, min_points=10).cluster(X)   # tuple of int

Same class, same constructor arguments, same ``cluster`` overloads and the same
exceptions as the SWIG binding: ``ValueError`` where upstream throws
std::invalid_argument, ``RuntimeError`` for std::runtime_error.  ``cluster(ndarray)``
converts its input to contiguous float64 exactly like the binding's IN_ARRAY2
typemap (swig/hpdbscan.i:27) and returns a tuple; ``cluster_array`` is the
numpy-native variant that keeps the input's element type and returns an int64
array.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .hdf5 import read_hdf5

_DTYPES = {
    np.dtype(np.float32): _lib.F32, np.dtype(np.float64): _lib.F64,
    np.dtype(np.int8): _lib.I8, np.dtype(np.int16): _lib.I16, np.dtype(np.int32): _lib.I32,
    np.dtype(np.int64): _lib.I64, np.dtype(np.uint8): _lib.U8, np.dtype(np.uint16): _lib.U16,
    np.dtype(np.uint32): _lib.U32, np.dtype(np.uint64): _lib.U64,
}


class HPDBSCAN:
    """HPDBSCAN(epsilon, min_points) -- upstream include/hpdbscan.h:288-298."""

    def __init__(self, epsilon: float, min_points: int):
        lib = _lib.load()
        if int(min_points) < 0:
            raise OverflowError("in method 'new_HPDBSCAN', argument 2 of type 'size_t'")
        h = ctypes.c_void_p()
        _lib.raise_for(lib.hpd_create(float(epsilon), int(min_points), ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self.epsilon = float(epsilon)
        self.min_points = int(min_points)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.hpd_destroy(h)
            self._h = None

    # arithmetic of the reference build being matched (see include/hpdbscan_gb300.h)
    def set_arith(self, cell_mode: int = _lib.CELL_RECIP, dist_mode: int = _lib.DIST_GCC_X86) -> None:
        _lib.raise_for(self._lib.hpd_set_arith(self._h, cell_mode, dist_mode))

    def set_tie_break(self, mode: int = _lib.TIE_EXACT) -> None:
        """TIE_EXACT (default): the single-thread reference's labels.  TIE_SMALLEST_ID:
        borders next to several clusters take the smallest cluster id among their core
        neighbours (faster; cores, noise and other borders unchanged)."""
        _lib.raise_for(self._lib.hpd_set_tie_break(self._h, mode))

    def set_tie_pass_limit(self, passes: int = 0) -> None:
        """Relaxation passes of the exact tie-break before HPD_ERR_TIMEOUT; 0: default."""
        _lib.raise_for(self._lib.hpd_set_tie_pass_limit(self._h, int(passes)))

    def set_tuning(self, sparse_queries: int = 0, dense_min_points: int = 0, greedy_tiles: int = 0) -> None:
        """Work decomposition of this handle's calls (labels do not depend on it; 0: the
        size-class table, then the built-in default)."""
        t = _lib.Tuning(int(sparse_queries), int(dense_min_points), int(greedy_tiles))
        _lib.raise_for(self._lib.hpd_set_tuning(self._h, ctypes.byref(t)))

    def set_diagnostics(self, flags: int = 0) -> None:
        """DIAG_COUNT_PAIRS: count the core test's distance evaluations (stats core_pairs)."""
        _lib.raise_for(self._lib.hpd_set_diagnostics(self._h, int(flags)))

    def debug_inject(self, what: int) -> None:
        """Test hook for the next call: INJECT_FAIL_ALLOC."""
        _lib.raise_for(self._lib.hpd_debug_inject(self._h, int(what)))

    def cluster(self, data, dataset: str | None = None, threads: int | None = None):
        """cluster(ndarray) | cluster(path, dataset[, threads]) -> tuple of int."""
        if isinstance(data, (str, bytes)):
            # HPDBSCAN::cluster(path, dataset[, threads]) (include/hpdbscan.h:300-356): the
            # dataset in its own element type, dispatched like the reference
            if dataset is None:
                raise TypeError("cluster(path, dataset[, threads]) needs the dataset name")
            path = data if isinstance(data, str) else data.decode()
            arr = read_hdf5(path, dataset.decode() if isinstance(dataset, bytes) else dataset)
            return tuple(self.cluster_array(arr).tolist())
        arr = np.ascontiguousarray(np.asarray(data, dtype=np.float64))
        return tuple(self.cluster_array(arr).tolist())

    def cluster_array(self, data) -> np.ndarray:
        """Labels (int64, input order) of an (n, d) array of any of the ten element types."""
        arr = np.ascontiguousarray(data)
        if arr.ndim != 2:
            raise ValueError("Array must have 2 dimensions")
        if arr.dtype not in _DTYPES:
            raise ValueError("Unsupported data set type")
        n, d = arr.shape
        out = np.empty(n, dtype=np.int64)
        rc = self._lib.hpd_cluster(self._h, arr.ctypes.data, n, d, _DTYPES[arr.dtype], 0, out.ctypes.data)
        _lib.raise_for(rc)
        return out

    def cluster_device(self, data_ptr: int, n: int, d: int, dtype, labels_ptr: int, stream: int = 0) -> None:
        """Cluster an (n, d) row-major array already in device memory into int64 labels."""
        code = _DTYPES[np.dtype(dtype)]
        rc = self._lib.hpd_cluster_device(self._h, ctypes.c_void_p(data_ptr), n, d, code,
                                          ctypes.c_void_p(labels_ptr), ctypes.c_void_p(stream or None))
        _lib.raise_for(rc)

    def stats(self) -> dict:
        st = _lib.Stats()
        _lib.raise_for(self._lib.hpd_get_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in _lib.Stats._fields_}
