"""Python surface of the upstream SWIG module on the GPU engine, and its errors."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_cluster_returns_tuple_of_int_like_swig(gpu, oracle):
    from hpdbscan_gb300 import HPDBSCAN
    rng = np.random.default_rng(0)
    x = rng.random((3000, 2)).astype(np.float32)
    got = HPDBSCAN(epsilon=0.03, min_points=5).cluster(x)
    assert isinstance(got, tuple) and all(isinstance(v, int) for v in got)
    # the binding converts to float64 before clustering (swig/hpdbscan.i:27)
    want = oracle.cluster(x.astype(np.float64), 0.03, 5, threads=1)
    assert np.array_equal(np.array(got), want)


def test_cluster_accepts_lists_and_noncontiguous(gpu, oracle):
    from hpdbscan_gb300 import HPDBSCAN
    rng = np.random.default_rng(1)
    x = rng.random((4000, 6))[:, ::2]  # non-contiguous float64 view
    got = HPDBSCAN(0.05, 4).cluster(x)
    want = oracle.cluster(np.ascontiguousarray(x), 0.05, 4, threads=1)
    assert np.array_equal(np.array(got), want)
    assert HPDBSCAN(0.5, 1).cluster([[0.0, 0.0], [0.1, 0.1], [3.0, 3.0]]) == (-1, -1, -3)


def test_empty_input(gpu):
    from hpdbscan_gb300 import HPDBSCAN
    assert HPDBSCAN(0.1, 2).cluster(np.zeros((0, 3))) == ()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_non_finite_rejected(gpu, dtype):
    from hpdbscan_gb300 import HPDBSCAN
    x = np.random.default_rng(2).random((100, 3)).astype(dtype)
    x[17, 1] = np.inf
    with pytest.raises(ValueError, match="non-finite"):
        HPDBSCAN(0.1, 2).cluster_array(x)


def test_shape_errors(gpu):
    from hpdbscan_gb300 import HPDBSCAN
    h = HPDBSCAN(0.1, 2)
    with pytest.raises(ValueError):
        h.cluster_array(np.zeros(10, np.float32))
    with pytest.raises(ValueError):
        h.cluster_array(np.zeros((10, 17), np.float32))
    with pytest.raises(ValueError):
        h.cluster_array(np.zeros((10, 0), np.float32))
    with pytest.raises(ValueError, match="Unsupported data set type"):
        h.cluster_array(np.zeros((10, 2), np.complex64))


def test_file_path_without_hdf5(gpu):
    from hpdbscan_gb300 import HPDBSCAN
    with pytest.raises(ValueError, match="Could not open"):
        HPDBSCAN(0.1, 2).cluster("/nonexistent/file.h5", "DATA")


def test_device_entry_point(gpu, oracle):
    """hpd_cluster_device on torch-owned device buffers."""
    torch = pytest.importorskip("torch")
    from hpdbscan_gb300 import HPDBSCAN, workloads
    w = workloads.blobs_100k(3, n=40_000)
    x = torch.from_numpy(w.points).cuda()
    out = torch.empty(len(w.points), dtype=torch.int64, device="cuda")
    h = HPDBSCAN(w.eps, w.min_points)
    h.cluster_device(x.data_ptr(), x.shape[0], x.shape[1], np.float32, out.data_ptr())
    want = oracle.cluster(w.points, w.eps, w.min_points, threads=1)
    assert np.array_equal(out.cpu().numpy(), want)
