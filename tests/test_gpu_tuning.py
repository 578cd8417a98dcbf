"""Work-decomposition tuning (hpd_set_tuning, hpd_set_tuning_table): labels never change.

The tuner (hpdbscan_gb300/tune.py) picks, per size class of the batch workload, how
many points a work item may hold for the core test's flat path, from how many points a
cell is connected through certified sub-cells, and how many tiles the tie-break's
greedy descent scans.  These only move work between code paths, so every setting
must give the labels of the built-in defaults.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SETTINGS = [(4, 64, 2), (16, 256, 12), (32, 32, 1), (0, 0, 0)]


@pytest.mark.parametrize("inst", [0, 3, 5, 11])
def test_tuning_keeps_labels(gpu, inst):
    from hpdbscan_gb300 import HPDBSCAN, workloads
    w = workloads.batch_instance(inst, n_max=200_000)
    want = HPDBSCAN(w.eps, w.min_points).cluster_array(w.points)
    for sq, dm, gt in SETTINGS:
        h = HPDBSCAN(w.eps, w.min_points)
        h.set_tuning(sq, dm, gt)
        assert np.array_equal(h.cluster_array(w.points), want), (sq, dm, gt)


def test_tuning_table_applies_and_keeps_labels(gpu):
    from hpdbscan_gb300 import HPDBSCAN, _lib, tune, workloads
    w = workloads.blobs_100k(seed=4, n=60_000)
    want = HPDBSCAN(w.eps, w.min_points).cluster_array(w.points)
    arr = (_lib.TuningEntry * 2)()
    arr[0].max_points, arr[0].dims, arr[0].tuning = 1000, 0, _lib.Tuning(4, 64, 2)
    arr[1].max_points, arr[1].dims, arr[1].tuning = 1 << 40, 3, _lib.Tuning(32, 32, 1)
    lib = gpu
    try:
        assert lib.hpd_set_tuning_table(arr, 2) == 0
        assert np.array_equal(HPDBSCAN(w.eps, w.min_points).cluster_array(w.points), want)
    finally:
        tune.clear_table()


def test_tuning_rejects_out_of_range(gpu):
    from hpdbscan_gb300 import HPDBSCAN
    h = HPDBSCAN(0.1, 4)
    with pytest.raises(ValueError):
        h.set_tuning(sparse_queries=33)
    with pytest.raises(ValueError):
        h.set_tuning(dense_min_points=8)
