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


def _smallest_root_labels(points, eps, exact):
    """Expected smallest-id labels from the exact ones: a border takes 1 + the
    smallest root among its core eps-neighbours (float32 d = 3: the squared distance
    is the sequential float sum, as in the engine's default arithmetic)."""
    from scipy.spatial import cKDTree
    eps2 = np.float32(eps) * np.float32(eps)
    core = np.flatnonzero(exact < 0)
    tree = cKDTree(points[core].astype(np.float64))
    want = exact.copy()
    border = np.flatnonzero(exact > 0)
    for b, cand in zip(border, tree.query_ball_point(points[border].astype(np.float64), float(eps) * 1.001)):
        c = core[np.asarray(cand, dtype=np.int64)]
        t = points[c] - points[b]
        sq = (t[:, 0] * t[:, 0] + t[:, 1] * t[:, 1]) + t[:, 2] * t[:, 2]
        roots = -exact[c[sq <= eps2]] - 1
        want[b] = roots.min() + 1
    return want


def test_gpu_smallest_id_tie_break(gpu):
    """HPD_TIE_SMALLEST_ID: cores, noise and single-cluster borders keep their exact
    labels; a border next to several clusters takes the smallest of their ids."""
    from hpdbscan_gb300 import _lib, workloads
    w = workloads.blobs_10m(seed=0, n=300_000)
    exact = engine(w.eps, w.min_points).cluster_array(w.points)
    h = engine(w.eps, w.min_points)
    h.set_tie_break(_lib.TIE_SMALLEST_ID)
    fast = h.cluster_array(w.points)
    assert h.stats()["n_ambiguous"] > 0
    assert np.array_equal(fast[exact <= 0], exact[exact <= 0])
    assert np.array_equal(fast == 0, exact == 0)
    assert np.array_equal(fast, _smallest_root_labels(w.points, w.eps, exact))
    h.set_tie_break(_lib.TIE_EXACT)
    assert np.array_equal(h.cluster_array(w.points), exact)
    with pytest.raises(ValueError):
        h.set_tie_break(7)


def test_gpu_stats_counts(gpu, oracle):
    """hpd_get_stats: cores and cells of the last call match the labels and the grid."""
    pts, eps, mp, labels = load_golden("blobs100k_s0")
    h = engine(eps, mp)
    assert np.array_equal(h.cluster_array(pts), labels)
    st = h.stats()
    assert st["n_core"] == int((labels < 0).sum())
    _, _, cells = oracle.cluster(pts, eps, mp, with_order=True)
    assert st["n_cells"] == len(np.unique(cells))


@pytest.mark.parametrize("d,dtype,k", [(2, np.float32, 0), (3, np.float32, 1), (4, np.float32, 2),
                                       (2, np.float64, 3), (3, np.float32, 4)])
def test_gpu_big_cells(gpu, oracle, d, dtype, k):
    """Cells of thousands of points (compact blobs, sigma ~ eps / 10) ringed by points at
    every distance: the box-certified counts, hits and pruning of big cells give the
    oracle's labels."""
    rng = np.random.default_rng(40 + k)
    eps = 0.01
    centres = rng.random((6, d)) * 0.5 + 0.25
    blobs = [c + rng.normal(0, eps * rng.uniform(0.05, 0.3), (int(rng.integers(2000, 9000)), d)) for c in centres]
    blobs[0] = centres[0] + rng.normal(0, eps * 0.05, (12000, d))  # one cell above the pruning size
    ring = np.concatenate([c + rng.uniform(-3 * eps, 3 * eps, (1500, d)) for c in centres])
    pts = np.concatenate(blobs + [ring, rng.random((3000, d))]).astype(dtype)
    pts = pts[rng.permutation(len(pts))]
    for mp in (4, 40, 400):
        want = oracle.cluster(pts, eps, mp, threads=1)
        assert np.array_equal(engine(eps, mp).cluster_array(pts), want), mp
