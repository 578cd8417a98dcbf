"""GB300-native DBSCAN engine with the interface of HPDBSCAN's single-node path.

``HPDBSCAN(epsilon, min_points).cluster(X)`` (or ``.cluster(path, dataset)`` for an
HDF5 file) mirrors the upstream Python module;
the computation runs in hand-written sm_103a CUDA kernels behind the C ABI in
include/hpdbscan_gb300.h (library: hpdbscan_gb300/libhpdbscan_gb300.so).
"""
from .hdf5 import read_hdf5, write_hdf5  # noqa: F401
from .hpdbscan import HPDBSCAN  # noqa: F401

__all__ = ["HPDBSCAN", "read_hdf5", "write_hdf5"]
