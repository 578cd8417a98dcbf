"""HDF5 files of the reference's file path: ``IO::read_hdf5`` / ``IO::write_hdf5``
(include/io.h:35-197) over the library's own HDF5 implementation (hpd_h5_read /
hpd_h5_write of include/hpdbscan_gb300.h; libhdf5 is not needed).

    >>> X = read_hdf5("data.h5", "DATA")          # (n, d) array in the file's element type
    >>> write_hdf5("data.h5", "CLUSTERS", labels)  # 1-D int64 dataset, created or overwritten

Errors are the reference's: ``ValueError`` for "Could not open <path>", "Could not open
dataset <name>", "Data in dataset <name> should be a matrix" and the unsupported element
types, ``RuntimeError`` for "Failed to read data" / "Failed to write data, ...".
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_NUMPY = {_lib.F32: np.float32, _lib.F64: np.float64, _lib.I8: np.int8, _lib.I16: np.int16, _lib.I32: np.int32,
          _lib.I64: np.int64, _lib.U8: np.uint8, _lib.U16: np.uint16, _lib.U32: np.uint32, _lib.U64: np.uint64}


def read_hdf5(path: str, dataset: str) -> np.ndarray:
    """The 2-D dataset ``dataset`` of the file ``path`` as a C-order array of its own element type."""
    lib = _lib.load()
    buf, n, d, dtype = ctypes.c_void_p(), ctypes.c_int64(), ctypes.c_int32(), ctypes.c_int32()
    rc = lib.hpd_h5_read(path.encode(), dataset.encode(), ctypes.byref(buf), ctypes.byref(n), ctypes.byref(d),
                         ctypes.byref(dtype))
    _lib.raise_for(rc)
    try:
        t = np.dtype(_NUMPY[dtype.value])
        count = n.value * d.value
        raw = (ctypes.c_char * (count * t.itemsize)).from_address(buf.value) if count else b""
        return np.frombuffer(raw, dtype=t, count=count).reshape(n.value, d.value).copy()
    finally:
        lib.hpd_h5_free(buf)


def write_hdf5(path: str, dataset: str, labels) -> None:
    """Writes ``labels`` (converted to int64) as the 1-D dataset ``dataset`` of ``path``."""
    arr = np.ascontiguousarray(np.asarray(labels, dtype=np.int64).reshape(-1))
    _lib.raise_for(_lib.load().hpd_h5_write(path.encode(), dataset.encode(), arr.ctypes.data, arr.size))
