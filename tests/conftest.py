import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: full-size workload")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build(ref=False)
    return pyoracle


@pytest.fixture(scope="session")
def engine_lib():
    """The engine's shared library, built in-tree if needed."""
    from hpdbscan_gb300 import _lib, build
    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(engine_lib):
    import ctypes
    n = ctypes.c_int(0)
    cudart = None
    for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
        try:
            cudart = ctypes.CDLL(name)
            break
        except OSError:
            continue
    if cudart is None or cudart.cudaGetDeviceCount(ctypes.byref(n)) != 0 or n.value < 1:
        pytest.fail("no CUDA device: GPU tests must run on a GPU host")
    return engine_lib


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    """(points, eps, min_points, labels) of one fixture; regenerated points are checked by hash."""
    import hashlib

    from hpdbscan_gb300 import workloads
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    if "points" in z:
        pts = z["points"]
    else:
        kind, seed = str(z["regen"]).split(":")
        assert kind == "blobs_100k"
        pts = workloads.blobs_100k(int(seed)).points
        digest = hashlib.sha256(np.ascontiguousarray(pts).tobytes()).hexdigest()
        assert digest == str(z["sha256"]), "regenerated points differ from the fixture's (numpy version?)"
    return pts, float(z["eps"]), int(z["min_points"]), z["labels"]
