"""Batched and served clustering on one GPU (include/hpdbscan_gb300.h: hpd_cluster_batch,
hpd_server_*).  No counterpart in the upstream project, which clusters one dataset
per call.

    labels = cluster_batch([(X1, eps1, minpts1), (X2, eps2, minpts2), ...])

    with Server(workers=8, budget_bytes=120 << 30) as srv:
        t = srv.submit(X, eps, min_points)      # returns at once
        labels = srv.wait(t)                    # int64 labels, input order

Every job's labels are exactly those of HPDBSCAN(eps, min_points).cluster_array(X).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_CODES = {np.dtype(np.float32): _lib.F32, np.dtype(np.float64): _lib.F64}


def _job(points, eps, min_points, deadline_ms=0.0):
    pts = np.ascontiguousarray(points)
    if pts.ndim != 2 or pts.dtype not in _CODES:
        raise ValueError("jobs take (n, d) float32 or float64 arrays")
    labels = np.empty(pts.shape[0], dtype=np.int64)
    j = _lib.Job()
    j.data = pts.ctypes.data
    j.n, j.d = pts.shape
    j.dtype = _CODES[pts.dtype]
    j.epsilon = float(eps)
    j.min_points = int(min_points)
    j.labels = labels.ctypes.data
    j.deadline_ms = float(deadline_ms)
    return j, pts, labels


_TABLE_LOADED = False


def _load_tuning_table():
    """Register the autotuner's size-class table (hpdbscan_gb300/tuning_table.json) once."""
    global _TABLE_LOADED
    if not _TABLE_LOADED:
        from . import tune
        tune.load_table()
        _TABLE_LOADED = True


def cluster_batch(items, workers: int = 8, with_stats: bool = False):
    """Labels of every (points, eps, min_points) item, clustered concurrently."""
    lib = _lib.load()
    _load_tuning_table()
    built = [_job(*it) for it in items]
    arr = (_lib.Job * len(built))(*[b[0] for b in built])
    rc = lib.hpd_cluster_batch(arr, len(built), workers)
    for j in arr:
        if j.status != 0:
            _lib.raise_for(j.status)
    if rc != 0:
        _lib.raise_for(rc)
    labels = [b[2] for b in built]
    if with_stats:
        return labels, [(j.queue_ms, j.run_ms) for j in arr]
    return labels


class Server:
    """Continuous-batching clustering server on the current GPU."""

    def __init__(self, workers: int = 8, budget_bytes: int = 120 << 30, reserve_points: int = 0,
                 reserve_dims: int = 3):
        self._lib = _lib.load()
        _load_tuning_table()
        h = ctypes.c_void_p()
        rc = self._lib.hpd_server_create(workers, budget_bytes, reserve_points, reserve_dims, ctypes.byref(h))
        if rc:
            raise RuntimeError(self._lib.hpd_server_last_error().decode())
        self._h = h
        self._pending = {}

    def submit(self, points, eps, min_points, deadline_ms: float = 0.0) -> int:
        """Queue a job; one still waiting for a worker deadline_ms after submission fails
        with HPD_ERR_TIMEOUT (TimeoutError from wait) without running."""
        job = _job(points, eps, min_points, deadline_ms)
        t = ctypes.c_int64()
        rc = self._lib.hpd_server_submit(self._h, ctypes.byref(job[0]), ctypes.byref(t))
        if rc:
            raise ValueError(self._lib.hpd_server_last_error().decode())
        self._pending[t.value] = job
        return t.value

    def done(self, ticket: int) -> bool:
        flag = ctypes.c_int32()
        self._lib.hpd_server_poll(self._h, ticket, ctypes.byref(flag))
        return bool(flag.value)

    def wait(self, ticket: int, with_stats: bool = False):
        job = self._pending.pop(ticket)
        status = self._lib.hpd_server_wait(self._h, ticket)
        if status == _lib.HPD_ERR_TIMEOUT:
            raise TimeoutError("job passed its deadline before a worker took it")
        if status:
            raise RuntimeError(f"job failed with status {status}")
        if with_stats:
            return job[2], job[0].queue_ms, job[0].run_ms
        return job[2]

    def close(self):
        if getattr(self, "_h", None):
            self._lib.hpd_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()
