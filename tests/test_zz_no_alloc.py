"""The allocation-free entry point (hpd_cluster_device_noalloc) against the regular
device entry point (hpd_cluster_device), through the C ABI.

hpd_cluster_device_noalloc serves callers that cannot call cudaMalloc: its scratch is
a fixed device array inside the library, so it takes at most 32768 points.  Two calls
in a row on different inputs must each give exactly the labels of the regular entry
point (the array keeps the previous call's contents), and oversized inputs must be
refused with a clear error.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _regular(torch, pts, eps, mp):
    from hpdbscan_gb300 import HPDBSCAN
    x = torch.from_numpy(pts).cuda()
    out = torch.empty(len(pts), dtype=torch.int64, device="cuda")
    HPDBSCAN(eps, mp).cluster_device(x.data_ptr(), pts.shape[0], pts.shape[1], pts.dtype, out.data_ptr())
    torch.cuda.synchronize()
    return x, out


def test_no_alloc_matches_regular_entry_point_twice(gpu):
    torch = pytest.importorskip("torch")
    from hpdbscan_gb300 import _lib, workloads
    lib = gpu
    cases = [
        workloads.blobs_100k(5, n=30_000),                      # float32, d = 3
        workloads.batch_instance(4, n_max=30_000),               # float32, d = 2
    ]
    f64 = workloads.batch_instance(0, n_max=20_000)              # d = 5, as float64
    inputs = [(w.points, w.eps, w.min_points) for w in cases] + [(f64.points.astype(np.float64), f64.eps, f64.min_points)]
    # the largest plans the 16 MiB array must hold, at exactly 32768 points: sixteen
    # float64 dimensions whose grid needs 64-bit cell ids, and four float32 dimensions
    # with one dense cell (sub-cell tables)
    rng = np.random.default_rng(7)
    inputs.append((rng.random((32768, 16)), 0.25, 4))
    dense = np.concatenate([0.5 + rng.standard_normal((30000, 4)) * 0.0025, rng.random((2768, 4))])
    inputs.append((np.ascontiguousarray(dense, dtype=np.float32), 0.05, 8))
    for pts, eps, mp in inputs:
        assert len(pts) <= 32768
        x, want = _regular(torch, pts, eps, mp)
        got = torch.full((len(pts),), -7, dtype=torch.int64, device="cuda")
        code = _lib.F32 if pts.dtype == np.float32 else _lib.F64
        rc = lib.hpd_cluster_device_noalloc(eps, mp, 0, 0, ctypes.c_void_p(x.data_ptr()), pts.shape[0],
                                            pts.shape[1], code, ctypes.c_void_p(got.data_ptr()), None)
        assert rc == 0, lib.hpd_noalloc_last_error()
        torch.cuda.synchronize()
        assert torch.equal(got, want)


def test_no_alloc_refuses_oversized_input(gpu):
    torch = pytest.importorskip("torch")
    lib = gpu
    x = torch.zeros((32769, 2), dtype=torch.float32, device="cuda")
    out = torch.empty(32769, dtype=torch.int64, device="cuda")
    rc = lib.hpd_cluster_device_noalloc(0.1, 4, 0, 0, ctypes.c_void_p(x.data_ptr()), 32769, 2, 0,
                                        ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 1
    assert b"32768" in lib.hpd_noalloc_last_error()
