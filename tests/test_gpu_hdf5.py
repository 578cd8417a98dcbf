"""The reference's file path end to end on the GPU: HPDBSCAN::cluster(path, dataset)
(include/hpdbscan.h:300-356) from Python and from the C++ header, and the command line
tool reading the input dataset and writing the labels into the HDF5 output file
(src/cli.cpp:84-119), each against the oracle.  Input files are laid out by
tests/h5_files.py as libhdf5 writes them; the labels the tool writes are read back by
that module's independent reader."""
import os
import subprocess

import numpy as np
import pytest

import h5_files as H

pytestmark = pytest.mark.gpu

DTYPES = [np.float32, np.float64, np.int8, np.int16, np.int32, np.int64, np.uint8, np.uint16, np.uint32, np.uint64]


def _blobs(dt, n=6000, seed=1):
    """Blob mixture scaled to the element type's range (integer grids for integer types)."""
    from hpdbscan_gb300 import workloads
    w = workloads.blobs_100k(seed, n=n)
    if np.dtype(dt).kind == "f":
        return w.points.astype(dt), w.eps, w.min_points
    return np.clip(np.round(w.points * 100), 0, 120).astype(dt), w.eps * 100, w.min_points


@pytest.mark.parametrize("fmt", ["earliest", "latest"])
@pytest.mark.parametrize("dt", DTYPES, ids=lambda t: np.dtype(t).name)
def test_python_cluster_path_matches_oracle(gpu, oracle, tmp_path, fmt, dt):
    from hpdbscan_gb300 import HPDBSCAN
    pts, eps, mp = _blobs(dt)
    p = str(tmp_path / "data.h5")
    H.write_matrix(p, pts, fmt=fmt, layout="chunked" if dt in (np.int16, np.float64) else "contiguous",
                   chunk=(1000, pts.shape[1]))
    got = HPDBSCAN(eps, mp).cluster(p, "DATA")
    assert isinstance(got, tuple)
    assert np.array_equal(np.array(got), oracle.cluster(pts, eps, mp, threads=1))


def test_python_cluster_path_errors(gpu, tmp_path):
    from hpdbscan_gb300 import HPDBSCAN
    h = HPDBSCAN(0.1, 4)
    with pytest.raises(ValueError, match="^Could not open "):
        h.cluster(str(tmp_path / "none.h5"), "DATA")
    p = str(tmp_path / "x.h5")
    H.write_matrix(p, np.zeros((5, 2), np.float32))
    with pytest.raises(ValueError, match="^Could not open dataset OTHER$"):
        h.cluster(p, "OTHER")
    H.write_matrix(p, np.zeros((5, 2), np.uint8), dtype_msg=H.dt_float(2))
    with pytest.raises(ValueError, match="^Unsupported floating point precision$"):
        h.cluster(p, "DATA")


def test_cpp_header_cluster_path(gpu, oracle, tmp_path):
    from conftest import ROOT
    from hpdbscan_gb300 import build
    exe = str(tmp_path / "cluster_demo")
    libdir = os.path.dirname(build.LIB)
    subprocess.run(["g++", "-std=c++11", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "cluster_demo.cpp"), "-o", exe, "-L", libdir,
                    "-lhpdbscan_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    pts, eps, mp = _blobs(np.uint16, n=8000, seed=2)
    p, out = str(tmp_path / "d.h5"), str(tmp_path / "l.i64")
    H.write_matrix(p, pts, name="grp/DATA", big=True)
    r = subprocess.run([exe, "--h5", p, "grp/DATA", repr(eps), str(mp), out], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout == "", r.stdout + r.stderr
    assert np.array_equal(np.fromfile(out, dtype=np.int64), oracle.cluster(pts, eps, mp, threads=1))
    r = subprocess.run([exe, "--h5", p, "DATA", repr(eps), str(mp), out], capture_output=True, text=True)
    assert r.stdout.strip() == "invalid_argument: Could not open dataset DATA"


def test_cli_reads_and_writes_hdf5(gpu, oracle, tmp_path):
    from hpdbscan_gb300 import build
    pts, eps, mp = _blobs(np.float32, n=20000, seed=3)
    p = str(tmp_path / "data.h5")
    H.write_matrix(p, pts)
    # upstream defaults: input dataset DATA, labels into CLUSTERS of the same file
    r = subprocess.run([build.CLI, "-m", str(mp), "-e", repr(eps), "-i", p, "-o", p], capture_output=True, text=True)
    assert r.returncode == 0 and r.stderr == "", r.stderr
    want = oracle.cluster(pts, eps, mp, threads=1)
    got = H.check_structure(p, ["CLUSTERS"])["CLUSTERS"]
    assert np.array_equal(got, want)
    # the points are untouched; a second run overwrites the labels in place
    from hpdbscan_gb300 import read_hdf5
    assert np.array_equal(read_hdf5(p, "DATA"), pts)
    out = str(tmp_path / "out.h5")
    r = subprocess.run([build.CLI, "-m", str(mp), "-e", repr(eps), "-i", p, "--input-dataset", "DATA", "-o", out,
                        "--output-dataset", "labels"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stderr == "", r.stderr
    assert np.array_equal(H.read_labels(out, "labels"), want)
    r = subprocess.run([build.CLI, "-i", p, "--input-dataset", "MISSING"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stderr.strip() == "Could not open dataset MISSING"
    r = subprocess.run([build.CLI, "-i", str(tmp_path / "none.h5")], capture_output=True, text=True)
    assert r.returncode == 0 and r.stderr.strip() == "Could not open " + str(tmp_path / "none.h5")
