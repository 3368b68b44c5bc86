"""The allocation-free solve (km_solve_noalloc) against the ordinary device solve (km_solve_dev).

km_solve_noalloc serves callers that cannot call cudaMalloc while solving (allocation would
synchronise the device, or an outside pool owns the device memory): its workspace is a fixed
8 MiB device array compiled into the library.  The calls below run back to back on the same
array, which keeps the previous call's contents: two calls in a row on one handle, then a call
on a handle of another shape, each compared with km_solve_dev on the same right-hand sides
(relative 1e-12; both run the same kernels in the same order, so they agree to the last bit in
practice).  Mixed handles are checked with FP64 refinement switched on, and in-place calls
(d_x == d_b) as well.  ACA handles are rejected.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _handle(n, level, rank, mixed=False, refine=0):
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    pts = uniform_points(n, 17)
    prec = K.KM_PREC_MIXED if mixed else K.KM_PREC_FP64
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, [1.0, 0.1, 1e-3], K.Matern32()), 0.0, rank,
                       K.FixedLevel(level), nystrom=True, precision=prec, refine_max_iter=refine)
    K.symmetricfactorize(hk)
    return hk


def _solve_pair(lib, hk, n, k, seed, in_place):
    """km_solve_dev and km_solve_noalloc on the same right-hand sides; returns both results."""
    import torch
    from kmhodlr import _lib as L
    b = torch.from_numpy(np.random.default_rng(seed).standard_normal((k, n))).cuda()
    x_ref = torch.empty_like(b)
    torch.cuda.synchronize()
    rc = lib.km_solve_dev(hk._h, C.c_void_p(b.data_ptr()), C.c_void_p(x_ref.data_ptr()), k)
    assert rc == L.KM_OK, lib.km_last_error(hk._h)
    if in_place:
        x_na = b.clone()
        src = x_na
    else:
        x_na = torch.full_like(b, float("nan"))
        src = b
    torch.cuda.synchronize()
    rc = lib.km_solve_noalloc(hk._h, C.c_void_p(src.data_ptr()), C.c_void_p(x_na.data_ptr()), k)
    assert rc == L.KM_OK, lib.km_last_error(hk._h)
    torch.cuda.synchronize()
    return x_ref.cpu().numpy(), x_na.cpu().numpy()


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("in_place", [False, True])
def test_noalloc_solve_matches_device_solve(lib, mixed, in_place):
    refine = 5 if mixed else 0
    first = _handle(8192, 5, 72, mixed, refine)
    second = _handle(4096, 4, 48, mixed, refine)
    for hk, n, k, seed in ((first, 8192, 4, 100), (first, 8192, 4, 101), (second, 4096, 7, 102)):
        xr, xn = _solve_pair(lib, hk, n, k, seed, in_place)
        assert np.all(np.isfinite(xn))
        assert np.linalg.norm(xn - xr) / np.linalg.norm(xr) < 1e-12
        if mixed:
            assert hk.stats().refine_residual <= 1e-10


def test_device_solve_in_place_refinement_matches_out_of_place(lib):
    """km_solve_dev with refinement in place (d_x == d_b) keeps the right-hand sides for the
    residual, so it gives the out-of-place result."""
    import torch
    from kmhodlr import _lib as L
    hk = _handle(4096, 4, 48, mixed=True, refine=5)
    n, k = 4096, 2
    b = torch.from_numpy(np.random.default_rng(7).standard_normal((k, n))).cuda()
    x = torch.empty_like(b)
    xb = b.clone()
    torch.cuda.synchronize()
    assert lib.km_solve_dev(hk._h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), k) == L.KM_OK
    assert lib.km_solve_dev(hk._h, C.c_void_p(xb.data_ptr()), C.c_void_p(xb.data_ptr()), k) == L.KM_OK
    torch.cuda.synchronize()
    xo, xi = x.cpu().numpy(), xb.cpu().numpy()
    assert np.linalg.norm(xi - xo) / np.linalg.norm(xo) < 1e-12
    assert hk.stats().refine_residual <= 1e-10


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


def test_noalloc_rejects_aca_handles(lib):
    import torch
    import kmhodlr as K
    from kmhodlr import _lib as L
    rng = np.random.default_rng(3)
    n = 1024
    pts = rng.standard_normal((n, 2))
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, [1.0, 1.0, 1.0], K.RatQuad()), 1e-12, 0, K.LogLevel(8))
    K.symmetricfactorize(hk)
    b = torch.ones((1, n), dtype=torch.float64, device="cuda")
    x = torch.empty_like(b)
    rc = lib.km_solve_noalloc(hk._h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), 1)
    assert rc == L.KM_ERR_UNSUPPORTED
    assert b"only Nystrom handles" in lib.km_last_error(hk._h)
