"""The oracle (C restatement) pinned against the upstream build, on the CPU.

* every golden fixture (labels produced by the upstream headers compiled with the
  upstream flags) is reproduced bit for bit in the default arithmetic mode;
* the known-answer sets really pin the arithmetic: each other mode disagrees;
* where the upstream build exists (this build host), fresh seeded inputs agree too,
  including the cell ids and the sorted order of the spatial index.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden


# The oracle walks every in-grid neighbour cell like the reference (up to 3^d per cell):
# on hidim_d16 that takes about 15 minutes (it agreed with the upstream labels when the
# fixture was made), too long for the CPU suite; the GPU tests check that fixture.
SLOW_FOR_ORACLE = {"hidim_d16"}


@pytest.mark.parametrize("name", [n for n in golden_names() if n not in SLOW_FOR_ORACLE])
def test_oracle_matches_golden(oracle, name):
    pts, eps, mp, labels = load_golden(name)
    got = oracle.cluster(pts, eps, mp, threads=1)
    assert np.array_equal(got, labels)


@pytest.mark.parametrize("name,modes", [
    ("kat_cells", [(1, 0)]),
    ("kat_dist_d3", [(0, 2)]),
    ("kat_dist_d4", [(0, 1), (0, 2)]),
    ("kat_dist_d5", [(0, 1), (0, 2)]),
    ("kat_dist64_d4", [(0, 1), (0, 2)]),
    ("kat_dist64_d5", [(0, 1), (0, 2)]),
])
def test_known_answers_discriminate_modes(oracle, name, modes):
    pts, eps, mp, labels = load_golden(name)
    for cell_mode, dist_mode in modes:
        got = oracle.cluster(pts, eps, mp, 1, cell_mode, dist_mode)
        assert not np.array_equal(got, labels), (cell_mode, dist_mode)


def test_multithreaded_oracle_core_set(oracle):
    """threads > 1 keeps core/noise flags and core labels (only borders may vary)."""
    pts, eps, mp, labels = load_golden("blobs100k_s0")
    got = oracle.cluster(pts, eps, mp, threads=4)
    assert np.array_equal(got < 0, labels < 0)
    assert np.array_equal(got == 0, labels == 0)
    assert np.array_equal(got[labels < 0], labels[labels < 0])


def test_oracle_errors(oracle):
    with pytest.raises(oracle.OracleError, match="epsilon needs to be positive"):
        oracle.cluster(np.zeros((3, 2), np.float32), 0.0, 2)
    bad = np.zeros((3, 2), np.float32)
    bad[1, 1] = np.nan
    with pytest.raises(oracle.OracleError, match="non-finite"):
        oracle.cluster(bad, 0.1, 2)


# --------------------------------------------------------------- upstream build
def _ref(oracle):
    if not oracle.ref_available():
        try:
            oracle.build(ref=True)
        except Exception:
            pass
    if not oracle.ref_available():
        pytest.skip("upstream sources not available on this host")


@pytest.mark.parametrize("seed,d,n,dtype", [
    (101, 2, 20000, np.float32), (102, 3, 30000, np.float32), (103, 4, 15000, np.float32),
    (104, 5, 12000, np.float32), (105, 3, 20000, np.float64), (106, 5, 8000, np.float64),
])
def test_oracle_matches_upstream_fresh(oracle, seed, d, n, dtype):
    _ref(oracle)
    from hpdbscan_gb300 import workloads
    rng = np.random.default_rng(seed)
    centres = rng.random((12, d))
    pts = workloads._mixture(rng, n, d, centres, np.full(12, 0.03), np.full(12, 1 / 12), 0.1).astype(dtype)
    eps, mp = 0.03 + 0.01 * (d - 2), 6
    want = oracle.ref_cluster(pts, eps, mp, threads=1)
    got = oracle.cluster(pts, eps, mp, threads=1)
    assert np.array_equal(got, want)


def test_index_order_matches_upstream(oracle):
    _ref(oracle)
    from hpdbscan_gb300 import workloads
    w = workloads.batch_instance(3, n_max=50_000)
    cells, order, dims, swapped = oracle.ref_index(w.points, w.eps)
    _, o_order, o_cells = oracle.cluster(w.points, w.eps, w.min_points, with_order=True)
    assert np.array_equal(order, o_order)
    assert np.array_equal(cells, o_cells)


@pytest.mark.slow
def test_oracle_matches_upstream_1m(oracle):
    _ref(oracle)
    from hpdbscan_gb300 import workloads
    w = workloads.blobs_10m(seed=3, n=1_000_000)
    want = oracle.ref_cluster(w.points, w.eps, w.min_points, threads=1)
    got = oracle.cluster(w.points, w.eps, w.min_points, threads=1)
    assert np.array_equal(got, want)
