"""GPU path vs the golden fixtures and the oracle, through the C ABI (bit-exact int64 labels)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu


def engine(eps, mp, cell_mode=0, dist_mode=0):
    from hpdbscan_gb300 import HPDBSCAN
    h = HPDBSCAN(eps, mp)
    h.set_arith(cell_mode, dist_mode)
    return h


@pytest.mark.parametrize("name", golden_names())
def test_gpu_matches_golden(gpu, name):
    pts, eps, mp, labels = load_golden(name)
    got = engine(eps, mp).cluster_array(pts)
    assert got.dtype == np.int64
    assert np.array_equal(got, labels), f"{int((got != labels).sum())} labels differ"


@pytest.mark.parametrize("name", ["kat_cells", "kat_dist_d3", "kat_dist_d4", "kat_dist_d5",
                                  "kat_dist64_d4", "kat_dist64_d5", "batch_0", "batch_3"])
@pytest.mark.parametrize("cell_mode,dist_mode", [(0, 0), (0, 1), (0, 2), (1, 0), (1, 1), (1, 2)])
def test_gpu_arith_modes_match_oracle(gpu, oracle, name, cell_mode, dist_mode):
    pts, eps, mp, _ = load_golden(name)
    want = oracle.cluster(pts, eps, mp, 1, cell_mode, dist_mode)
    got = engine(eps, mp, cell_mode, dist_mode).cluster_array(pts)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("seed", [0, 1, 2, 3, 4])
def test_gpu_blobs_100k_seeds(gpu, oracle, seed):
    from hpdbscan_gb300 import workloads
    w = workloads.blobs_100k(seed)
    want = oracle.cluster(w.points, w.eps, w.min_points, threads=1)
    assert np.array_equal(engine(w.eps, w.min_points).cluster_array(w.points), want)


@pytest.mark.parametrize("i", range(8, 28))
def test_gpu_batch_instances(gpu, oracle, i):
    """Uneven sizes, d in 2..5, per-instance eps / minPoints (batch workload)."""
    from hpdbscan_gb300 import workloads
    w = workloads.batch_instance(i, n_max=60_000)
    want = oracle.cluster(w.points, w.eps, w.min_points, threads=1)
    got = engine(w.eps, w.min_points).cluster_array(w.points)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("i", [30, 31, 32])
def test_gpu_float64(gpu, oracle, i):
    from hpdbscan_gb300 import workloads
    w = workloads.batch_instance(i, n_max=40_000)
    pts = w.points.astype(np.float64)
    want = oracle.cluster(pts, w.eps, w.min_points, threads=1)
    assert np.array_equal(engine(w.eps, w.min_points).cluster_array(pts), want)


def test_gpu_skewed_density(gpu, oracle):
    from hpdbscan_gb300 import workloads
    w = workloads.skewed_2d(seed=1, n=300_000)
    want = oracle.cluster(w.points, w.eps, w.min_points, threads=1)
    assert np.array_equal(engine(w.eps, w.min_points).cluster_array(w.points), want)


def test_gpu_blobs_1m_many_ties(gpu, oracle):
    """1M points of the 10M workload's distribution: > 1,000 borders next to 2+ clusters."""
    from hpdbscan_gb300 import workloads
    w = workloads.blobs_10m(seed=0, n=1_000_000)
    want = oracle.cluster(w.points, w.eps, w.min_points, threads=1)
    h = engine(w.eps, w.min_points)
    got = h.cluster_array(w.points)
    assert h.stats()["n_ambiguous"] > 100
    assert np.array_equal(got, want), f"{int((got != want).sum())} labels differ"


def test_gpu_repeatable_and_reusable(gpu):
    """Same handle, different sizes back to back, identical results on repeat."""
    from hpdbscan_gb300 import workloads
    h = engine(0.02, 8)
    a = workloads.blobs_100k(0, n=50_000).points
    b = workloads.blobs_100k(1).points
    ra = h.cluster_array(a)
    rb = h.cluster_array(b)
    assert np.array_equal(h.cluster_array(a), ra)
    assert np.array_equal(h.cluster_array(b), rb)


def test_gpu_input_not_modified(gpu):
    from hpdbscan_gb300 import workloads
    pts = workloads.blobs_100k(0, n=10_000).points
    before = pts.copy()
    engine(0.02, 8).cluster_array(pts)
    assert np.array_equal(pts, before)
