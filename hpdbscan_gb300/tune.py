"""Autotuner of the engine's work decomposition for batched and served clustering.

    python -m hpdbscan_gb300.tune [--per-class 3] [--out hpdbscan_gb300/tuning_table.json]

Batched and served work mixes jobs of very different shapes (the batch workload:
1e3..1e6 points, 2..5 dimensions).  Three choices of the engine's work decomposition
depend on the shape, and none changes a label:

* ``sparse_queries``    work items of at most this many points take the core test's
                        flat path (one candidate list, every query per candidate);
* ``dense_min_points``  cells with at least this many points are connected through
                        certified sub-cells instead of pairwise tests;
* ``greedy_tiles``      candidate tiles a work item of the tie-break's greedy descent
                        scans before it settles for its own position.

For each size class (points in [1e3, 1e4), [1e4, 1e5), [1e5, 1e6], times d = 2..5) the
tuner clusters sample instances of the batch workload and picks the parameters one at
a time (coordinate descent from the built-in defaults) by the median device time of
the whole clustering, checking that every setting gives the same labels.  Above the
largest class the library's own values apply (for three or more dimensions: 16, 64
and 12, measured on the 10M-point 3-D workload).  The table
is written as JSON; ``load_table`` registers it with the library
(``hpd_set_tuning_table``), after which every call without a tuning of its own --
batch and served jobs included -- uses the entry of its size class.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics

import numpy as np

from . import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning_table.json")
DEFAULTS = {"sparse_queries": 8, "dense_min_points": 128, "greedy_tiles": 6}
CANDIDATES = {"sparse_queries": [4, 8, 16, 32], "dense_min_points": [64, 128, 256], "greedy_tiles": [2, 4, 6, 12]}
CLASSES = [(max_n, d) for max_n in (10_000, 100_000, 1_000_000) for d in (2, 3, 4, 5)]


def load_table(path: str = TABLE) -> bool:
    """Register a tuning table with the library; False when there is none."""
    if not os.path.exists(path):
        return False
    with open(path) as f:
        rows = json.load(f)["entries"]
    arr = (_lib.TuningEntry * len(rows))()
    for e, r in zip(arr, rows):
        e.max_points = int(r["max_points"])
        e.dims = int(r["dims"])
        e.tuning = _lib.Tuning(int(r["sparse_queries"]), int(r["dense_min_points"]), int(r["greedy_tiles"]))
    rc = _lib.load().hpd_set_tuning_table(arr, len(rows))
    _lib.raise_for(rc)
    return True


def clear_table() -> None:
    _lib.raise_for(_lib.load().hpd_set_tuning_table(None, 0))


def _samples(per_class: int, limit: int = 4000):
    """Batch-workload instances grouped by size class (the first per_class of each)."""
    from . import workloads
    picked = {c: [] for c in CLASSES}
    for i in range(limit):
        # the instance's shape is drawn first, so draw it cheaply before generating points
        r = np.random.default_rng(1_000_000 + i)
        n = int(np.exp(r.uniform(np.log(1e3), np.log(1_000_000))))
        d = int(r.integers(2, 6))
        cls = next(c for c in CLASSES if n <= c[0] and d == c[1])
        if len(picked[cls]) < per_class:
            picked[cls].append(workloads.batch_instance(i))
        if all(len(v) >= per_class for v in picked.values()):
            break
    return picked


def _time(w, tuning, repeats):
    from .hpdbscan import HPDBSCAN
    h = HPDBSCAN(w.eps, w.min_points)
    h.set_tuning(**tuning)
    labels = h.cluster_array(w.points)  # warm-up (and the labels to compare)
    ms = []
    for _ in range(repeats):
        h.cluster_array(w.points)
        ms.append(h.stats()["total_ms"])
    return statistics.median(ms), labels


def tune(per_class: int = 3, repeats: int = 3, log=print):
    clear_table()
    entries, report = [], []
    for (max_n, d), insts in _samples(per_class).items():
        best = dict(DEFAULTS)

        def cost(t):
            total, labs = 0.0, []
            for w in insts:
                ms, lab = _time(w, t, repeats)
                total += ms
                labs.append(lab)
            return total, labs

        base_ms, base_labels = cost(best)
        cur = base_ms
        for name, values in CANDIDATES.items():
            for v in values:
                if v == best[name]:
                    continue
                trial = dict(best, **{name: v})
                ms, labs = cost(trial)
                if not all(np.array_equal(a, b) for a, b in zip(labs, base_labels)):
                    raise AssertionError(f"labels changed with {trial} on class ({max_n}, {d})")
                if ms < cur:
                    cur, best = ms, trial
        entries.append({"max_points": max_n, "dims": d, **best})
        report.append({"max_points": max_n, "dims": d, "instances": [len(w.points) for w in insts],
                       "default_ms": round(base_ms, 3), "tuned_ms": round(cur, 3), **best})
        log(f"class n<={max_n:>9,} d={d}: default {base_ms:8.3f} ms -> tuned {cur:8.3f} ms  {best}")
    return entries, report


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--per-class", type=int, default=3)
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--out", default=TABLE)
    args = ap.parse_args()
    entries, report = tune(args.per_class, args.repeats)
    with open(args.out, "w") as f:
        json.dump({"entries": entries, "report": report,
                   "note": "sum over the class's sample instances of the median device time per clustering"},
                  f, indent=1)
    print(f"wrote {args.out}")


if __name__ == "__main__":
    main()
