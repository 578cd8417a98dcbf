"""Seeded synthetic point sets with the shapes of the benchmark workloads.

The upstream project benchmarks on downloaded datasets (bremen_small, twitter_small,
iris; benchmarks/download_datasets.py) that are not available offline, so these
generators stand in for them with fixed seeds:

* ``blobs_100k``    100,000 x 3 float32, 20 isotropic Gaussian blobs (centres U[0,1]^3,
                    sigma 0.02, equal weights) + 10 % uniform noise; eps 0.02, minPts 8.
* ``blobs_10m``     10,000,000 x 3 float32, 200 blobs (sigma log-U[0.005, 0.03], weights
                    Dirichlet(1)) + 5 % uniform noise; eps 0.005, minPts 16.
* ``skewed_2d``     N x 2 float32 in [0,1]^2, 1,000 anisotropic rotated Gaussians (axis
                    sigmas log-U[1e-4, 5e-3]) with Zipf(1.1) weights + 2 % noise;
                    eps 1e-3, minPts 32 (50M points at full size).
* ``batch_instance``  one instance of the 4,096-instance batch (n log-U[1e3, 1e6], d in
                    {2..5}, 5-100 blobs, sigma log-U[0.005, 0.05], 5 % noise,
                    eps U[0.005, 0.03], minPts U{4..32}); seed = instance id.
* ``serve_trace``   Poisson arrivals at 200 jobs/s for 60 s, each job a blob mixture of
                    n log-U[1e4, 5e6] points, d in {2,3,4}, eps U[0.002, 0.02],
                    minPts in {8,16,32}.

Every generator shuffles its points so that input order carries no structure.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class Workload:
    name: str
    points: np.ndarray  # (n, d) float32, C-contiguous
    eps: float
    min_points: int


def _mixture(rng, n, d, centres, sigmas, weights, noise_frac, rot=None, clip=False):
    n_noise = int(round(n * noise_frac))
    n_blob = n - n_noise
    counts = rng.multinomial(n_blob, weights)
    parts = []
    for b, c in enumerate(counts):
        if c == 0:
            continue
        z = rng.standard_normal((c, d)) * sigmas[b]
        if rot is not None:
            z = z @ rot[b].T
        parts.append(z + centres[b])
    parts.append(rng.random((n_noise, d)))
    pts = np.concatenate(parts, axis=0)
    if clip:
        np.clip(pts, 0.0, 1.0, out=pts)
    pts = pts[rng.permutation(n)]
    return np.ascontiguousarray(pts, dtype=np.float32)


def blobs_100k(seed: int = 0, n: int = 100_000) -> Workload:
    rng = np.random.default_rng(seed)
    k, d = 20, 3
    centres = rng.random((k, d))
    pts = _mixture(rng, n, d, centres, np.full(k, 0.02), np.full(k, 1.0 / k), 0.10)
    return Workload(f"blobs_100k(seed={seed},n={n})", pts, 0.02, 8)


def blobs_10m(seed: int = 0, n: int = 10_000_000) -> Workload:
    rng = np.random.default_rng(seed)
    k, d = 200, 3
    centres = rng.random((k, d))
    sigmas = np.exp(rng.uniform(np.log(0.005), np.log(0.03), k))
    weights = rng.dirichlet(np.ones(k))
    pts = _mixture(rng, n, d, centres, sigmas, weights, 0.05)
    return Workload(f"blobs_10m(seed={seed},n={n})", pts, 0.005, 16)


def skewed_2d(seed: int = 0, n: int = 50_000_000) -> Workload:
    rng = np.random.default_rng(seed)
    k, d = 1000, 2
    centres = rng.random((k, d))
    sig = np.exp(rng.uniform(np.log(1e-4), np.log(5e-3), (k, d)))
    ang = rng.uniform(0, 2 * np.pi, k)
    rot = np.stack([np.stack([np.cos(ang), -np.sin(ang)], 1), np.stack([np.sin(ang), np.cos(ang)], 1)], 1)
    w = 1.0 / np.arange(1, k + 1) ** 1.1
    w = w[rng.permutation(k)]
    w /= w.sum()
    pts = _mixture(rng, n, d, centres, sig, w, 0.02, rot=rot, clip=True)
    return Workload(f"skewed_2d(seed={seed},n={n})", pts, 1e-3, 32)


def batch_instance(i: int, n_max: int = 1_000_000) -> Workload:
    rng = np.random.default_rng(1_000_000 + i)
    n = int(np.exp(rng.uniform(np.log(1e3), np.log(n_max))))
    d = int(rng.integers(2, 6))
    k = int(rng.integers(5, 101))
    centres = rng.random((k, d))
    sigmas = np.exp(rng.uniform(np.log(0.005), np.log(0.05), k))
    weights = rng.dirichlet(np.ones(k))
    pts = _mixture(rng, n, d, centres, sigmas, weights, 0.05)
    eps = float(rng.uniform(0.005, 0.03))
    mp = int(rng.integers(4, 33))
    return Workload(f"batch_instance({i})", pts, eps, mp)


@dataclasses.dataclass
class Job:
    arrival_s: float
    n: int
    d: int
    eps: float
    min_points: int
    seed: int

    def points(self) -> np.ndarray:
        rng = np.random.default_rng(self.seed)
        k = int(rng.integers(5, 51))
        centres = rng.random((k, self.d))
        sigmas = np.exp(rng.uniform(np.log(0.005), np.log(0.05), k))
        weights = rng.dirichlet(np.ones(k))
        return _mixture(rng, self.n, self.d, centres, sigmas, weights, 0.05)


def serve_trace(seed: int = 0, rate: float = 200.0, duration_s: float = 60.0, n_max: int = 5_000_000):
    rng = np.random.default_rng(seed)
    t, jobs = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration_s:
            break
        n = int(np.exp(rng.uniform(np.log(1e4), np.log(n_max))))
        jobs.append(Job(t, n, int(rng.choice([2, 3, 4])), float(rng.uniform(0.002, 0.02)),
                        int(rng.choice([8, 16, 32])), int(rng.integers(0, 2**31))))
    return jobs
