"""Full-size workloads against the upstream single-thread build, bit for bit.

The upstream HPDBSCAN::cluster<float>(data, n, d, threads=1) takes minutes on these
inputs, so its labels are pinned by tests/golden/make_fullsize.py into
tests/golden/fullsize/<set>.npz: the sha256 of the input the generator makes, the
sha256 of the full int64 label vector, the core / border / noise counts and, for
diagnostics, every border point with cores of several clusters within eps together
with its upstream label.  A test here regenerates the input, clusters it on the GPU
and requires the identical label vector (same sha256); on a mismatch it reports which
kind of point differs.

Sets: the 10M-point 3-D benchmark workload (eps 0.005, minPoints 16) and the skewed
2-D density at 1M and 5M points (eps 1e-3, minPoints 32; the upstream single-thread
run takes 312 s and 2.4 h on these).
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

FULL = os.path.join(GOLDEN, "fullsize")


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _load(name, make):
    z = np.load(os.path.join(FULL, name + ".npz"))
    w = make()
    assert _sha(w.points) == str(z["points_sha256"]), "regenerated points differ from the fixture's (numpy version?)"
    return w, z


def _check(got, z):
    if _sha(got.astype(np.int64)) == str(z["labels_sha256"]):
        return
    amb, want = z["amb_index"], z["amb_label"]
    detail = (f"core {(got < 0).sum()} vs {int(z['n_core'])}, border {(got > 0).sum()} vs {int(z['n_border'])}, "
              f"noise {(got == 0).sum()} vs {int(z['n_noise'])}; "
              f"multi-cluster borders differing {(got[amb] != want).sum()} of {len(amb)}")
    pytest.fail("labels differ from the upstream single-thread build: " + detail)


@pytest.fixture(scope="module")
def blobs10m(gpu):
    from hpdbscan_gb300 import HPDBSCAN, workloads
    w, z = _load("blobs10m_s0", lambda: workloads.blobs_10m(seed=0))
    h = HPDBSCAN(w.eps, w.min_points)
    got = h.cluster_array(w.points)
    again = h.cluster_array(w.points)
    return w, z, got, again


def test_blobs10m_bit_exact(blobs10m):
    _, z, got, _ = blobs10m
    _check(got, z)


def test_blobs10m_repeatable(blobs10m):
    _, _, got, again = blobs10m
    assert np.array_equal(got, again)


def test_skewed1m_bit_exact(gpu):
    from hpdbscan_gb300 import HPDBSCAN, workloads
    w, z = _load("skewed1m_s0", lambda: workloads.skewed_2d(seed=0, n=1_000_000))
    _check(HPDBSCAN(w.eps, w.min_points).cluster_array(w.points), z)


def test_skewed5m_bit_exact(gpu):
    from hpdbscan_gb300 import HPDBSCAN, workloads
    w, z = _load("skewed5m_s0", lambda: workloads.skewed_2d(seed=0, n=5_000_000))
    _check(HPDBSCAN(w.eps, w.min_points).cluster_array(w.points), z)
