"""The allocation-free solve (km_solve_noalloc) against the ordinary device solve (km_solve_dev).

km_solve_noalloc serves callers that cannot call cudaMalloc while solving (allocation would
synchronise the device, or an outside pool owns the device memory): its workspace is a fixed
8 MiB device array compiled into the library.  Two calls in a row must both match the ordinary
entry point, since the shared array keeps the previous call's contents.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _handle(n, level, rank):
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    pts = uniform_points(n, 17)
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, [1.0, 0.1, 1e-3], K.Matern32()), 0.0, rank,
                       K.FixedLevel(level), nystrom=True)
    K.symmetricfactorize(hk)
    return hk


def test_noalloc_solve_matches_device_solve_twice(lib):
    import torch
    from kmhodlr import _lib as L
    n, k = 8192, 4
    hk = _handle(n, 5, 72)
    for call in range(2):
        b = torch.from_numpy(np.random.default_rng(100 + call).standard_normal((k, n))).cuda()
        x_ref = torch.empty_like(b)
        x_na = torch.full_like(b, float("nan"))
        torch.cuda.synchronize()
        rc = lib.km_solve_dev(hk._h, C.c_void_p(b.data_ptr()), C.c_void_p(x_ref.data_ptr()), k)
        assert rc == L.KM_OK, lib.km_last_error(hk._h)
        rc = lib.km_solve_noalloc(hk._h, C.c_void_p(b.data_ptr()), C.c_void_p(x_na.data_ptr()), k)
        assert rc == L.KM_OK, lib.km_last_error(hk._h)
        torch.cuda.synchronize()
        xr, xn = x_ref.cpu().numpy(), x_na.cpu().numpy()
        assert np.all(np.isfinite(xn))
        assert np.linalg.norm(xn - xr) / np.linalg.norm(xr) < 1e-12


def test_noalloc_rejects_oversized_requests(lib):
    import torch
    from kmhodlr import _lib as L
    n = 8192
    hk = _handle(n, 5, 72)
    k = 128  # 63 slots * 72 * 128 * 2 doubles already exceed 8 MiB
    b = torch.zeros((k, n), dtype=torch.float64, device="cuda")
    x = torch.empty_like(b)
    rc = lib.km_solve_noalloc(hk._h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), k)
    assert rc == L.KM_ERR_BAD_ARG
    assert b"fixed array holds" in lib.km_last_error(hk._h)
