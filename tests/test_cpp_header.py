"""include/hpdbscan.h: the upstream HPDBSCAN class interface over the C ABI."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "cluster_demo.cpp")


@pytest.fixture(scope="module")
def demo(engine_lib, tmp_path_factory):
    from hpdbscan_gb300 import build
    out = str(tmp_path_factory.mktemp("cpp") / "cluster_demo")
    libdir = os.path.dirname(build.LIB)
    cmd = ["g++", "-std=c++11", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), SRC, "-o", out,
           "-L", libdir, "-lhpdbscan_gb300", f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True)
    return out


def test_header_compiles_as_cpp11_and_links(demo):
    assert os.path.exists(demo)


def test_constructor_throws_invalid_argument(demo):
    r = subprocess.run([demo, "--bad-eps"], capture_output=True, text=True)
    assert r.returncode == 0
    assert "invalid_argument: epsilon needs to be positive" in r.stdout


@pytest.mark.gpu
def test_cpp_class_matches_oracle(gpu, oracle, demo, tmp_path):
    from hpdbscan_gb300 import workloads
    w = workloads.blobs_100k(4, n=20_000)
    pts_file, lab_file = tmp_path / "p.f32", tmp_path / "l.i64"
    w.points.tofile(pts_file)
    r = subprocess.run([demo, str(pts_file), str(len(w.points)), "3", repr(w.eps), str(w.min_points), str(lab_file)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "file: Could not open /nonexistent/data.h5" in r.stdout
    got = np.fromfile(lab_file, dtype=np.int64)
    assert np.array_equal(got, oracle.cluster(w.points, w.eps, w.min_points, threads=1))
