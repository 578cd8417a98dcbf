"""Generates the golden fixtures from the UPSTREAM build (oracle/_ref/libhpdref.so).

    python tests/golden/make_golden.py        # needs the upstream sources to build _ref

Each fixture holds the input points (or, for the two 100k sets, the sha256 of the
points that hpdbscan_gb300.workloads regenerates), epsilon, minPoints and the
labels the upstream HPDBSCAN::cluster<T>(data, n, d, threads=1) returned.  The
upstream build is the reference's own headers compiled with its own flags
(g++ -std=c++11 -Ofast -fopenmp) on x86-64, whose arithmetic is reciprocal cell
coordinates and the SSE2 partial-sum order of squared distances; manifest.json
records this.

Sets:
  blobs100k_s{0,1}   100,000 x 3 f32 blob mixture, eps 0.02, minPts 8
  batch_{i}          eight batch-workload instances (d = 2..5, n <= 30,000)
  skewed_60k         skewed 2-D density, 60,000 points
  f64_blobs          30,000 x 3 float64 (the Python binding's element type)
  kat_dist_d{2..5}   isolated point pairs at distance ~eps: each pair clusters
                     (minPts 2) iff the squared distance rounds <= eps^2, chosen
                     where the candidate summation orders disagree
  kat_cells          coordinates on cell boundaries, where x * (1/eps) and
                     x / eps round to different cells
  edge_*             edge cases: all-negative dimension (the max-init quirk),
                     duplicates, one point, minPts 0 / 1 / > n, one big cell
  int_<type>_d{2,3}  the eight integer element types (upstream instantiations), with
                     coordinates and eps chosen so that the squared distances wrap
                     around and EPS2 overflows the narrow types
  dims_d1, dims_d8   one dimension (with a cell of ~12,000 points) and eight
                     dimensions (the generic paths past d = 5)
  big_cells_d{2,3}   compact blobs (sigma eps/20) in cells of up to ~70,000 points,
                     ringed by points at every distance: cells this full take the
                     box-pruned queries and the finer sub-cell split
  hidim_d{6,12,16}   blob mixtures in 6, 12 and 16 dimensions (12 and 16 with 64-bit
                     cell ids; the upstream build enumerates up to 3^d neighbour cells
                     per cell and takes minutes on hidim_d16)

    python tests/golden/make_golden.py [name-prefix ...]   # all fixtures, or those named
"""
from __future__ import annotations

import hashlib
import json
import os
import platform
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hpdbscan_gb300 import workloads as wl  # noqa: E402
from oracle import pyoracle as po  # noqa: E402


def sha(points: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(points).tobytes()).hexdigest()


def save(name, points, eps, minpts, store_points=True, regen=None):
    labels = po.ref_cluster(points, eps, minpts, threads=1)
    meta = dict(eps=np.float32(eps), min_points=np.int64(minpts), sha256=sha(points),
                shape=np.array(points.shape), dtype=str(points.dtype))
    if store_points:
        meta["points"] = points
    if regen:
        meta["regen"] = regen
    np.savez_compressed(os.path.join(HERE, name + ".npz"), labels=labels, **meta)
    print(f"{name}: n={len(labels)} clusters={len(np.unique(np.abs(labels[labels != 0])))} "
          f"core={(labels < 0).sum()} border={(labels > 0).sum()} noise={(labels == 0).sum()}")


def kat_dist(d: int, dtype, seed: int, n_pairs: int = 20000):
    """Isolated pairs at distance ~eps whose within-test depends on the summation order."""
    rng = np.random.default_rng(seed)
    eps = np.float32(0.01)
    spacing = 5.0 * float(eps)
    side = int(np.ceil(n_pairs ** (1.0 / d)))
    grid = np.stack(np.unravel_index(np.arange(n_pairs), (side,) * d), 1).astype(np.float64) * spacing
    u = rng.standard_normal((n_pairs, d))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    # the threshold is EPS2 = fl32(eps * eps) converted to the element type
    radius = np.sqrt(np.float64(np.float32(eps * eps)))
    rel = 1.5e-7 if dtype == np.float32 else 3e-16
    scale = 1.0 + rng.uniform(-rel, rel, (n_pairs, 1))
    p = grid + rng.uniform(0, spacing / 4, (n_pairs, d)) + 0.5
    q = p + u * radius * scale
    pts = np.empty((2 * n_pairs, d), dtype=dtype)
    pts[0::2] = p
    pts[1::2] = q
    # keep the pairs on which the candidate orders disagree, plus some others
    within = {}
    for mode in (po.DIST_GCC_X86, po.DIST_SEQ, po.DIST_SEQ_FMA):
        lab = po.cluster(pts, float(eps), 2, 1, po.CELL_RECIP, mode)
        within[mode] = (lab[0::2] < 0)
    differ = (within[0] != within[1]) | (within[0] != within[2]) | (within[1] != within[2])
    keep = differ | (rng.random(n_pairs) < 0.005)
    idx = np.flatnonzero(keep)
    sel = np.empty((2 * len(idx), d), dtype=dtype)
    sel[0::2] = pts[2 * idx]
    sel[1::2] = pts[2 * idx + 1]
    return sel, float(eps), int(differ.sum())


def kat_cells(seed: int = 5):
    """Coordinates on cell boundaries: x - min within an ulp of k * eps."""
    rng = np.random.default_rng(seed)
    eps = np.float32(0.0137)
    n = 6000
    k = rng.integers(1, 60, n).astype(np.float32)
    x = (k * eps).astype(np.float32)
    x = np.nextafter(x, np.where(rng.random(n) < 0.5, np.float32(0), np.float32(10))).astype(np.float32)
    y = rng.random(n).astype(np.float32) * np.float32(0.8)
    pts = np.stack([x, y], 1).astype(np.float32)
    pts[0] = (0.0, 0.0)  # pins min at 0 in both dimensions
    return pts, float(eps)


def big_cells(d: int, seed: int):
    """A blob of 70,000 points with sigma eps/20 (one cell holds most of it), smaller
    compact blobs, a ring of points within 3 eps of every centre and uniform noise."""
    rng = np.random.default_rng(seed)
    eps = 0.01
    centres = rng.random((4, d)) * 0.5 + 0.25
    blobs = [centres[0] + rng.normal(0, eps / 20, (70000, d))]
    blobs += [c + rng.normal(0, eps * 0.2, (int(rng.integers(3000, 9000)), d)) for c in centres[1:]]
    ring = np.concatenate([c + rng.uniform(-3 * eps, 3 * eps, (1500, d)) for c in centres])
    pts = np.concatenate(blobs + [ring, rng.random((2000, d))]).astype(np.float32)
    return pts[rng.permutation(len(pts))], eps


def dims_case(d: int, seed: int):
    """Blob mixture in d dimensions; for d = 1 one blob is compact enough to fill a
    single cell with ~12,000 points."""
    rng = np.random.default_rng(seed)
    eps = 0.0005 if d == 1 else 0.08
    centres = rng.random((8, d))
    sig = np.full(8, eps * 0.6)
    n = [3000] * 8
    if d == 1:
        sig[0], n[0] = eps * 0.05, 12000
    blobs = [c + rng.normal(0, s, (k, d)) for c, s, k in zip(centres, sig, n)]
    pts = np.concatenate(blobs + [rng.random((2000, d))]).astype(np.float32)
    return pts[rng.permutation(len(pts))], eps


def hidim_case(d: int, seed: int):
    """Six Gaussian blobs (two of them side by side), a shell of fringe points just
    outside each blob (borders), points between the side-by-side pair and uniform noise,
    in d dimensions; eps spans a quarter to a tenth of the unit extent, and for d = 16
    the first dimension is twice as wide, so the grid has more than 2^32 cells."""
    rng = np.random.default_rng(seed)
    eps, sig, n_blob, n_noise, wide = {6: (0.08, 0.35, 3000, 2000, 1.0), 12: (0.1, 0.2, 500, 500, 1.0),
                                       16: (0.25, 0.15, 400, 150, 2.0)}[d]
    fringe = {6: (0.6, 1.1), 12: (0.3, 0.9), 16: (0.3, 0.9)}[d]
    ext = np.ones(d)
    ext[0] = wide
    centres = rng.random((6, d)) * ext * 0.9 + 0.05
    v = rng.standard_normal(d)
    centres[1] = centres[0] + v / np.linalg.norm(v) * 2.2 * eps * np.sqrt(d) * sig
    blobs = [c + rng.normal(0, eps * sig, (n_blob, d)) for c in centres]
    radius = eps * sig * np.sqrt(d)
    for c in centres:
        u = rng.standard_normal((n_blob // 10, d))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        blobs.append(c + u * (radius + eps * rng.uniform(*fringe, (len(u), 1))))
    blobs.append((centres[0] + centres[1]) / 2 + rng.normal(0, eps * 0.15, (40, d)))
    pts = np.concatenate(blobs + [rng.random((n_noise, d)) * ext]).astype(np.float32)
    return pts[rng.permutation(len(pts))], eps


def main():
    if not po.ref_available():
        po.build(ref=True)
    os.makedirs(HERE, exist_ok=True)
    only = sys.argv[1:]
    if only:  # regenerate only the named fixtures
        global save
        keep_save = save

        def save(name, *a, **k):  # noqa: F811
            if any(name.startswith(o) for o in only):
                keep_save(name, *a, **k)
    for s in (0, 1):
        w = wl.blobs_100k(seed=s)
        save(f"blobs100k_s{s}", w.points, w.eps, w.min_points, store_points=False, regen=f"blobs_100k:{s}")
    for i in range(8):
        w = wl.batch_instance(i, n_max=30_000)
        save(f"batch_{i}", w.points, w.eps, w.min_points)
    w = wl.skewed_2d(seed=0, n=60_000)
    save("skewed_60k", w.points, w.eps, w.min_points)
    w = wl.blobs_100k(seed=2, n=30_000)
    save("f64_blobs", w.points.astype(np.float64), w.eps, w.min_points)
    for d in (2, 3, 4, 5):
        pts, eps, nd = kat_dist(d, np.float32, seed=10 + d)
        print(f"  kat_dist_d{d}: {nd} discriminating pairs")
        save(f"kat_dist_d{d}", pts, eps, 2)
    for d in (4, 5):
        pts, eps, nd = kat_dist(d, np.float64, seed=20 + d)
        print(f"  kat_dist64_d{d}: {nd} discriminating pairs")
        save(f"kat_dist64_d{d}", pts, eps, 2)
    pts, eps = kat_cells()
    save("kat_cells", pts, eps, 3)
    rng = np.random.default_rng(7)
    neg = (rng.random((3000, 3)) - 2.0).astype(np.float32)   # every coordinate negative
    save("edge_negative", neg, 0.05, 4)
    dup = np.repeat(rng.random((300, 2)).astype(np.float32), 7, axis=0)
    save("edge_duplicates", dup, 0.01, 5)
    save("edge_one_point", np.array([[0.25, 0.5]], np.float32), 0.1, 1)
    small = rng.random((2000, 3)).astype(np.float32)
    save("edge_minpts0", small, 0.05, 0)
    save("edge_minpts1", small, 0.05, 1)
    save("edge_minpts_big", small, 0.05, 5000)
    save("edge_one_cell", small, 10.0, 50)
    rng = np.random.default_rng(11)
    for dt, lo, hi, eps in [(np.int8, -128, 127, 30.0), (np.uint8, 0, 255, 9.5), (np.int16, -3000, 3000, 90.0),
                            (np.uint16, 0, 60000, 1500.0), (np.int32, -100000, 100000, 4000.0),
                            (np.uint32, 0, 4000000, 90000.0), (np.int64, -10**6, 10**6, 30000.0),
                            (np.uint64, 0, 10**7, 2e5)]:
        for d in (2, 3):
            c = rng.integers(lo, hi, (8, d))
            pts = np.clip(c[rng.integers(0, 8, 3000)] + rng.normal(0, eps, (3000, d)), lo, hi).astype(dt)
            save(f"int_{np.dtype(dt).name}_d{d}", pts, eps, 6)
    for d in (1, 8):
        pts, eps = dims_case(d, seed=70 + d)
        save(f"dims_d{d}", pts, eps, 10)
    for d in (2, 3):
        pts, eps = big_cells(d, seed=60 + d)
        save(f"big_cells_d{d}", pts, eps, 40)
    for d in (6, 12, 16):
        if not only or any(f"hidim_d{d}".startswith(o) for o in only):
            pts, eps = hidim_case(d, seed=80 + d)
            save(f"hidim_d{d}", pts, eps, 8)
    manifest = {
        "reference_build": "upstream include/*.h via oracle/Makefile: g++ -std=c++11 -Ofast -fopenmp",
        "compiler": subprocess.run(["g++", "--version"], capture_output=True, text=True).stdout.splitlines()[0],
        "machine": platform.machine(),
        "cell_mode": "recip",
        "dist_mode": "gcc_x86",
        "threads": 1,
    }
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main()
