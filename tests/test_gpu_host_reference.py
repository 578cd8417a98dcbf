"""The engine against the upstream build made on THIS host, whichever host it is.

The reference's labels depend on how GCC compiled it (-Ofast): on x86-64 the squared
distances follow the SSE2 partial-sum order, on aarch64 NEON lanes accumulated with
fused multiply-adds, and out-of-range float -> integer conversions differ.  Here the
upstream headers are compiled on the host running the tests (from the upstream
checkout, or from the unmodified copy `make -C oracle stage` leaves in oracle/_ref),
a known-answer probe picks the engine's arithmetic mode that reproduces that build on
every known-answer set (pairs at distance ~eps where the summation orders disagree;
coordinates on cell boundaries), and the mode must be the one the host's architecture
names.  That mode is then checked bit for bit on blob mixtures, float64, the integer
element types and a 1M-point slab of the 10M workload, and the C restatement in the
same mode is checked against the host build too.
"""
import platform

import numpy as np
import pytest

from conftest import golden_names, load_golden

pytestmark = pytest.mark.gpu

HOST_MODE = {"x86_64": 0, "aarch64": 3}  # HPD_DIST_GCC_X86, HPD_DIST_GCC_AARCH64
KAT = [n for n in golden_names() if n.startswith("kat_")]


@pytest.fixture(scope="module")
def host_ref(gpu):
    from oracle import pyoracle
    if not pyoracle.ref_sources_available():
        pytest.skip("upstream sources neither checked out nor staged on this host")
    if platform.machine() not in HOST_MODE:
        pytest.skip(f"no arithmetic mode for {platform.machine()}")
    pyoracle.build(ref=True)
    return pyoracle, HOST_MODE[platform.machine()]


def _engine(pts, eps, mp, mode):
    from hpdbscan_gb300 import HPDBSCAN
    h = HPDBSCAN(eps, mp)
    h.set_arith(0, mode)
    return h.cluster_array(pts)


def test_probe_selects_the_host_mode(host_ref):
    po, mode = host_ref
    matching = {0, 1, 2, 3}
    for name in KAT:
        pts, eps, mp, _ = load_golden(name)
        ref = po.ref_cluster(pts, eps, mp, threads=1)
        matching &= {m for m in range(4) if np.array_equal(_engine(pts, eps, mp, m), ref)}
    assert mode in matching, f"modes reproducing the host build on every KAT set: {sorted(matching)}"


@pytest.mark.parametrize("name", [n for n in golden_names() if n.startswith(("kat_", "int_", "blobs100k", "batch_",
                                                                               "f64", "edge_", "dims_", "skewed"))])
def test_host_build_bit_exact(host_ref, name):
    po, mode = host_ref
    pts, eps, mp, _ = load_golden(name)
    ref = po.ref_cluster(pts, eps, mp, threads=1)
    assert np.array_equal(_engine(pts, eps, mp, mode), ref)
    assert np.array_equal(po.cluster(pts, eps, mp, threads=1, dist_mode=mode), ref)


@pytest.mark.slow
def test_host_build_bit_exact_1m_slab(host_ref):
    from hpdbscan_gb300 import workloads
    po, mode = host_ref
    w = workloads.blobs_10m(seed=0)
    x = w.points[:, 0]
    pts = np.ascontiguousarray(w.points[(x >= 0.45) & (x < 0.55)])
    ref = po.ref_cluster(pts, w.eps, w.min_points, threads=1)
    assert np.array_equal(_engine(pts, w.eps, w.min_points, mode), ref)
