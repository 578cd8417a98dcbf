"""Pins the full-size workloads to the UPSTREAM single-thread build (oracle/_ref/libhpdref.so).

    python tests/golden/make_fullsize.py [blobs10m_s0] [skewed1m_s0] [skewed5m_s0]

Writes tests/golden/fullsize/<set>.npz.  The single-thread upstream run takes minutes
to an hour per set, too long for a test, so each fixture stores what a test needs to
prove bit-exact labels without rerunning it:

* ``points_sha256``  sha256 of the regenerated input (hpdbscan_gb300.workloads), so a
                     generator change is reported as such;
* ``labels_sha256``  sha256 of the full int64 label vector in input order, as upstream
                     HPDBSCAN::cluster<float>(data, n, d, threads=1) returns it;
* counts of core / border / noise points and of clusters;
* ``amb_index`` / ``amb_label``  every border point with core points of two or more
                     clusters within eps (a float64 k-d tree query with a 1e-5 relative
                     margin), with its upstream label: the points the tie-break decides,
                     listed for diagnostics when the hash differs.

Sets (all seed 0):
  blobs10m_s0   10,000,000 x 3 float32 blob mixture, eps 0.005, minPts 16
  skewed1m_s0   1,000,000 x 2 float32 skewed density, eps 1e-3, minPts 32
  skewed5m_s0   5,000,000 x 2 float32 skewed density, eps 1e-3, minPts 32
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hpdbscan_gb300 import workloads as wl  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

OUT = os.path.join(HERE, "fullsize")  # apart from the per-point fixtures of make_golden.py

SETS = {
    "blobs10m_s0": lambda: wl.blobs_10m(seed=0),
    "skewed1m_s0": lambda: wl.skewed_2d(seed=0, n=1_000_000),
    "skewed5m_s0": lambda: wl.skewed_2d(seed=0, n=5_000_000),
}


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def multi_cluster_borders(points: np.ndarray, labels: np.ndarray, eps: float) -> np.ndarray:
    """Border points with cores of at least two clusters within eps (diagnostic list)."""
    from scipy.spatial import cKDTree
    core = np.flatnonzero(labels < 0)
    border = np.flatnonzero(labels > 0)
    tree = cKDTree(points[core].astype(np.float64))
    out = []
    step = 1 << 16
    for s in range(0, len(border), step):
        b = border[s:s + step]
        hits = tree.query_ball_point(points[b].astype(np.float64), r=eps * (1 + 1e-5))
        for p, nb in zip(b, hits):
            if len(nb) > 1 and len(np.unique(labels[core[nb]])) > 1:
                out.append(p)
    return np.asarray(out, dtype=np.int64)


def make(name: str) -> None:
    w = SETS[name]()
    t0 = time.time()
    labels = po.ref_cluster(w.points, w.eps, w.min_points, threads=1)
    secs = time.time() - t0
    amb = multi_cluster_borders(w.points, labels, w.eps)
    os.makedirs(OUT, exist_ok=True)
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"),
        workload=w.name, eps=np.float32(w.eps), min_points=np.int64(w.min_points),
        points_sha256=sha(w.points), labels_sha256=sha(labels.astype(np.int64)),
        n_core=np.int64((labels < 0).sum()), n_border=np.int64((labels > 0).sum()),
        n_noise=np.int64((labels == 0).sum()),
        n_clusters=np.int64(len(np.unique(-labels[labels < 0]))),
        amb_index=amb, amb_label=labels[amb], ref_seconds_1thread=np.float64(secs))
    print(f"{name}: {w.name} upstream 1 thread {secs:.1f} s; core {(labels < 0).sum()} "
          f"border {(labels > 0).sum()} noise {(labels == 0).sum()}; multi-cluster borders {len(amb)}")


if __name__ == "__main__":
    po.build(ref=True)
    for nm in sys.argv[1:] or ["blobs10m_s0", "skewed1m_s0"]:
        make(nm)
