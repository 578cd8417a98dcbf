"""Cluster one of the seeded workloads on the GPU and print the phase timings.

    python -m hpdbscan_gb300.run [--workload blobs_10m|blobs_100k|skewed_2d] [--n N] [--repeat R]

Used to profile the engine on a fixed input (e.g. under ncu) and as a quick check
that the library runs on a machine.
"""
from __future__ import annotations

import argparse
import json
import time

from . import HPDBSCAN, workloads


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="blobs_10m", choices=["blobs_10m", "blobs_100k", "skewed_2d"])
    ap.add_argument("--n", type=int, default=None)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--repeat", type=int, default=1)
    args = ap.parse_args()
    gen = getattr(workloads, args.workload)
    w = gen(seed=args.seed, n=args.n) if args.n else gen(seed=args.seed)
    h = HPDBSCAN(w.eps, w.min_points)
    for _ in range(args.repeat):
        t0 = time.perf_counter()
        labels = h.cluster_array(w.points)
        wall = time.perf_counter() - t0
        st = h.stats()
        st["wall_ms"] = 1000 * wall
        st["clusters"] = int(len(set(abs(int(v)) for v in labels[labels != 0][:1_000_000])))
        print(json.dumps({"workload": w.name, **{k: (round(v, 4) if isinstance(v, float) else v)
                                                  for k, v in st.items()}}), flush=True)


if __name__ == "__main__":
    main()
