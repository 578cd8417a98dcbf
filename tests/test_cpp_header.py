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


def test_io_dataset_roundtrip_on_cpu(demo, tmp_path):
    """IO::read_hdf5 -> Dataset (shape, element type, points) and IO::write_hdf5 of
    Clusters, through the library's own HDF5 implementation (no GPU needed)."""
    import h5_files as H
    pts = (np.arange(30, dtype=np.int16).reshape(10, 3) * 7)
    src, dst = str(tmp_path / "in.h5"), str(tmp_path / "out.h5")
    H.write_matrix(src, pts, name="grp/DATA")
    r = subprocess.run([demo, "--io-roundtrip", src, "grp/DATA", dst], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "shape 10 3 type 3"  # HPD_I16
    assert np.array_equal(H.read_labels(dst, "CLUSTERS"), np.arange(10) % 7 - 3)
    r = subprocess.run([demo, "--io-roundtrip", src, "MISSING", dst], capture_output=True, text=True)
    assert r.stdout.strip() == "invalid_argument: Could not open dataset MISSING"


@pytest.mark.gpu
def test_cluster_dataset_overload(gpu, oracle, demo, tmp_path):
    """HPDBSCAN::cluster<T>(Dataset&, threads) on a Dataset from IO::read_hdf5, labels
    written back with IO::write_hdf5; a mismatched element type is rejected."""
    import h5_files as H
    from hpdbscan_gb300 import workloads
    w = workloads.blobs_100k(5, n=15_000)
    src, dst = str(tmp_path / "in.h5"), str(tmp_path / "out.h5")
    H.write_matrix(src, w.points)
    r = subprocess.run([demo, "--io-cluster", src, "DATA", repr(w.eps), str(w.min_points), dst],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "invalid_argument: Dataset element type differs" in r.stdout
    want = oracle.cluster(w.points, w.eps, w.min_points, threads=1)
    assert np.array_equal(H.read_labels(dst, "CLUSTERS"), want)
