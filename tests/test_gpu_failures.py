"""Failure paths of the engine, made on the host or with bounded device loops only.

* The exact tie-break relaxes the reference's provisional labels pass by pass; its
  pass count is bounded by the handle's limit.  With a limit of one pass on an input
  that needs more, the call returns HPD_ERR_TIMEOUT; the same handle then clusters
  correctly.  (The upstream error surface is exceptions only, include/hpdbscan.h:
  288-298; here a status code plus hpd_last_error().)
* An allocation failure: HPD_INJECT_FAIL_ALLOC fails the first device allocation of
  the next call on the host, without attempting it: HPD_ERR_NOMEM, handle still usable.
* A serving deadline: a job still queued past its deadline completes with
  HPD_ERR_TIMEOUT without running, and the server keeps serving.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tied(workloads):
    """A slab of the 10M-point workload whose borders need the relaxation passes."""
    w = workloads.blobs_10m(seed=0)
    x = w.points[:, 0]
    sel = w.points[(x >= 0.45) & (x < 0.55)]
    return np.ascontiguousarray(sel), w.eps, w.min_points


def _cluster_rc(h, pts):
    from hpdbscan_gb300 import _lib
    out = np.empty(len(pts), np.int64)
    code = _lib.F32 if pts.dtype == np.float32 else _lib.F64
    rc = h._lib.hpd_cluster(h._h, pts.ctypes.data, pts.shape[0], pts.shape[1], code, 0, out.ctypes.data)
    return rc, out


def test_tie_pass_limit_times_out_then_handle_recovers(gpu, oracle):
    from hpdbscan_gb300 import HPDBSCAN, _lib, workloads
    pts, eps, mp = _tied(workloads)
    h = HPDBSCAN(eps, mp)
    want = h.cluster_array(pts)
    assert h.stats()["tie_iterations"] > 1, "input must need more than one relaxation pass"
    h.set_tie_pass_limit(1)
    rc, _ = _cluster_rc(h, pts)
    assert rc == _lib.HPD_ERR_TIMEOUT
    assert "tie-break" in h._lib.hpd_last_error().decode()
    h.set_tie_pass_limit(0)
    rc, got = _cluster_rc(h, pts)
    assert rc == _lib.HPD_OK
    assert np.array_equal(got, want)
    assert np.array_equal(got, oracle.cluster(pts, eps, mp, threads=1))


def test_allocation_failure_then_handle_recovers(gpu, oracle):
    from hpdbscan_gb300 import HPDBSCAN, _lib, workloads
    w = workloads.blobs_100k(seed=1, n=50_000)
    h = HPDBSCAN(w.eps, w.min_points)  # fresh handle: its first call must allocate
    h.debug_inject(_lib.INJECT_FAIL_ALLOC)
    rc, _ = _cluster_rc(h, w.points)
    assert rc == _lib.HPD_ERR_NOMEM
    with pytest.raises(MemoryError):
        h.debug_inject(_lib.INJECT_FAIL_ALLOC)
        h.cluster_array(w.points)
    rc, got = _cluster_rc(h, w.points)
    assert rc == _lib.HPD_OK
    assert np.array_equal(got, oracle.cluster(w.points, w.eps, w.min_points, threads=1))


def test_device_entry_point_allocation_failure(gpu):
    torch = pytest.importorskip("torch")
    from hpdbscan_gb300 import HPDBSCAN, _lib, workloads
    w = workloads.blobs_100k(seed=2, n=20_000)
    x = torch.from_numpy(w.points).cuda()
    out = torch.empty(len(w.points), dtype=torch.int64, device="cuda")
    h = HPDBSCAN(w.eps, w.min_points)
    h.debug_inject(_lib.INJECT_FAIL_ALLOC)
    rc = h._lib.hpd_cluster_device(h._h, ctypes.c_void_p(x.data_ptr()), len(w.points), 3, _lib.F32,
                                   ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _lib.HPD_ERR_NOMEM
    h.cluster_device(x.data_ptr(), len(w.points), 3, np.float32, out.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(out.cpu(), torch.from_numpy(h.cluster_array(w.points)))


def test_server_deadline(gpu):
    from hpdbscan_gb300 import HPDBSCAN, workloads
    from hpdbscan_gb300.serve import Server
    big = workloads.blobs_10m(seed=0, n=3_000_000)
    small = workloads.blobs_100k(seed=3, n=20_000)
    with Server(workers=1, budget_bytes=64 << 30) as srv:
        t_big = srv.submit(big.points, big.eps, big.min_points)
        # queued behind the big job on the only worker: past its deadline before it starts
        t_late = srv.submit(small.points, small.eps, small.min_points, deadline_ms=0.001)
        t_ok = srv.submit(small.points, small.eps, small.min_points)
        srv.wait(t_big)
        with pytest.raises(TimeoutError):
            srv.wait(t_late)
        got = srv.wait(t_ok)
    assert np.array_equal(got, HPDBSCAN(small.eps, small.min_points).cluster_array(small.points))
