"""Batched and served clustering give every job exactly its standalone labels."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _items(count, n_max=40_000, f64_every=5):
    from hpdbscan_gb300 import workloads
    items = []
    for i in range(count):
        w = workloads.batch_instance(100 + i, n_max=n_max)
        pts = w.points.astype(np.float64) if i % f64_every == 0 else w.points
        items.append((pts, w.eps, w.min_points))
    return items


def _alone(items):
    from hpdbscan_gb300 import HPDBSCAN
    return [HPDBSCAN(eps, mp).cluster_array(pts) for pts, eps, mp in items]


def test_batch_matches_standalone_and_oracle(gpu, oracle):
    from hpdbscan_gb300.serve import cluster_batch
    items = _items(40)
    got = cluster_batch(items, workers=8)
    want = _alone(items)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)
    for (pts, eps, mp), g in list(zip(items, got))[:8]:
        assert np.array_equal(g, oracle.cluster(pts, eps, mp, threads=1))


def test_server_results_same_alone_and_in_the_mix(gpu):
    """Jobs arriving while others run (Poisson arrivals) get their standalone labels."""
    from hpdbscan_gb300.serve import Server
    items = _items(30, n_max=100_000)
    want = _alone(items)
    rng = np.random.default_rng(0)
    gaps = rng.exponential(0.004, len(items))
    tickets = [None] * len(items)
    with Server(workers=6, budget_bytes=8 << 30) as srv:
        def submit():
            for i, it in enumerate(items):
                time.sleep(gaps[i])
                tickets[i] = srv.submit(*it)
        th = threading.Thread(target=submit)
        th.start()
        th.join()
        got = [srv.wait(t) for t in tickets]
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_server_tiny_budget_runs_one_at_a_time(gpu):
    from hpdbscan_gb300.serve import Server
    items = _items(6, n_max=20_000)
    want = _alone(items)
    with Server(workers=4, budget_bytes=1) as srv:
        ts = [srv.submit(*it) for it in items]
        got = [srv.wait(t, with_stats=True) for t in ts]
    for (g, q, r), w in zip(got, want):
        assert np.array_equal(g, w)
        assert r > 0


def test_server_rejects_bad_job(gpu):
    from hpdbscan_gb300.serve import Server
    with Server(workers=1) as srv:
        with pytest.raises(ValueError, match="epsilon"):
            srv.submit(np.zeros((10, 2), np.float32), -1.0, 3)


def test_batch_large_instances_identical_and_repeatable(gpu):
    """Instances of up to 1M points (dense cells, deep union-find trees): concurrent batch
    labels equal standalone labels, and standalone labels are the same run to run."""
    from hpdbscan_gb300 import workloads
    from hpdbscan_gb300.serve import cluster_batch
    items = []
    for i in range(48):
        w = workloads.batch_instance(i)
        items.append((w.points, w.eps, w.min_points))
    got = cluster_batch(items, workers=8)
    want = _alone(items)
    again = _alone(items)
    for k, (g, w, w2) in enumerate(zip(got, want, again)):
        assert np.array_equal(w, w2), k
        assert np.array_equal(g, w), k
