"""The hpdbscan command line tool: upstream flags, report format, exit code 0."""
import os
import subprocess

import numpy as np
import pytest


@pytest.fixture(scope="module")
def cli(engine_lib):
    from hpdbscan_gb300 import build
    assert os.path.exists(build.CLI)
    return build.CLI


def test_help_lists_the_upstream_flags(cli):
    out = subprocess.run([cli, "-h"], capture_output=True, text=True)
    assert out.returncode == 0
    for flag in ("-m, --minPoints", "-e, --epsilon", "-t, --threads", "-i, --input", "-o, --output",
                 "--input-dataset", "--output-dataset"):
        assert flag in out.stdout


def test_errors_go_to_stderr_with_exit_code_zero(cli, tmp_path):
    r = subprocess.run([cli, "--bogus"], capture_output=True, text=True)
    assert r.returncode == 0 and "Could not parse command line" in r.stderr
    r = subprocess.run([cli, "-e", "-1", "-i", str(tmp_path / "x.npy")], capture_output=True, text=True)
    assert r.returncode == 0 and "epsilon needs to be positive" in r.stderr


@pytest.mark.gpu
def test_cli_clusters_npy_file(gpu, oracle, cli, tmp_path):
    from hpdbscan_gb300 import workloads
    w = workloads.blobs_100k(6, n=30_000)
    src, dst = tmp_path / "points.npy", tmp_path / "labels.npy"
    np.save(src, w.points)
    r = subprocess.run([cli, "-m", str(w.min_points), "-e", repr(w.eps), "-i", str(src), "-o", str(dst)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.load(dst)
    want = oracle.cluster(w.points, w.eps, w.min_points, threads=1)
    assert got.dtype == np.int64 and np.array_equal(got, want)
    lines = r.stdout.splitlines()
    for head in ("Computing cell space", "\tDBSCAN...", "Summary...", "\tClusters:", "\tCore points:", "Total time:"):
        assert any(l.startswith(head) for l in lines), head
    summary = {l.split(":")[0].strip(): l.split(":")[1].strip() for l in lines if l.startswith("\t") and ":" in l
               and "[OK]" not in l}
    assert int(summary["Clusters"]) == len(np.unique(np.abs(want[want != 0])))
    assert int(summary["Noise points"]) == int((want == 0).sum())
    assert int(summary["Core points"]) == int((want < 0).sum())
