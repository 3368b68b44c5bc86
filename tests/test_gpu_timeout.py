"""Bounded device waits that run out, made to do so on purpose (km_set_wait_limit(h, 0): every
such wait gives up at its first poll, as if the flag it waits for were never set).

* The mixed-form node factorisation (dataflow flags between warps of a node): km_factorize
  returns KM_ERR_TIMEOUT.
* The grid-wide ACA kernel (grid barriers between the CTAs of an 8192 x 8192 block, n = 16384):
  km_assemble returns KM_ERR_TIMEOUT.
In both cases the same handle, with the default limit restored, assembles and factorises again
and gives the results of a fresh handle bit for bit.  No GPU fault or hang is involved: a wait
that gives up marks its status word and the kernel runs to its end.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _create(lib, precision):
    from kmhodlr import _lib as L
    h = C.c_void_p()
    cfg = L.KmConfig(device=0, precision=precision, hbm_budget_fraction=0.8, refine_max_iter=0, refine_tol=0.0)
    assert lib.km_create(C.byref(cfg), C.byref(h)) == L.KM_OK
    return h


def _assemble(lib, h, pts, params, kid, method, tol, rank, kind, level):
    from kmhodlr import hodlr as KH
    p = np.ascontiguousarray(params, dtype=np.float64)
    x = np.ascontiguousarray(pts, dtype=np.float64)
    return lib.km_assemble(h, KH._dp(x), len(pts), kid, KH._dp(p), 3, method, tol, rank, kind, level)


def _solve_logdet(lib, h, rhs):
    from kmhodlr import hodlr as KH
    b = np.asfortranarray(rhs)
    x = np.empty_like(b, order="F")
    ld = C.c_double()
    assert lib.km_solve(h, KH._dp(b), KH._dp(x), b.shape[1]) == 0, lib.km_last_error(h)
    assert lib.km_logdet(h, C.byref(ld)) == 0
    return x, ld.value


def test_node_flag_wait_runs_out_then_the_handle_recovers(lib):
    from kmhodlr import _lib as L
    from kmhodlr.data import uniform_points
    n = 8192
    pts = uniform_points(n, 61)
    rhs = np.random.default_rng(62).standard_normal((n, 2))
    args = ([1.0, 0.1, 1e-3], L.KM_KERNEL_MATERN32, L.KM_METHOD_NYSTROM, 0.0, 72, L.KM_LEVEL_FIXED, 5)
    h = _create(lib, L.KM_PREC_MIXED)
    assert _assemble(lib, h, pts, *args) == L.KM_OK
    assert lib.km_set_wait_limit(h, 0) == L.KM_OK
    assert lib.km_factorize(h) == L.KM_ERR_TIMEOUT
    assert b"bounded wait" in lib.km_last_error(h)
    assert lib.km_set_wait_limit(h, -1) == L.KM_OK
    assert _assemble(lib, h, pts, *args) == L.KM_OK
    assert lib.km_factorize(h) == L.KM_OK, lib.km_last_error(h)
    x, ld = _solve_logdet(lib, h, rhs)
    fresh = _create(lib, L.KM_PREC_MIXED)
    assert _assemble(lib, fresh, pts, *args) == L.KM_OK
    assert lib.km_factorize(fresh) == L.KM_OK
    x0, ld0 = _solve_logdet(lib, fresh, rhs)
    assert ld == ld0 and np.array_equal(x, x0)
    lib.km_destroy(h)
    lib.km_destroy(fresh)


def test_aca_grid_barrier_runs_out_then_the_handle_recovers(lib):
    from kmhodlr import _lib as L
    from kmhodlr.data import uniform_points
    n = 16384
    pts = uniform_points(n, 99)
    rhs = np.random.default_rng(98).standard_normal((n, 1))
    args = ([1.0, 0.2, 1e-2], L.KM_KERNEL_RATQUAD, L.KM_METHOD_ACA, 1e-10, 0, L.KM_LEVEL_LOG, 8)
    h = _create(lib, L.KM_PREC_FP64)
    assert lib.km_set_wait_limit(h, 0) == L.KM_OK
    assert _assemble(lib, h, pts, *args) == L.KM_ERR_TIMEOUT
    assert b"grid barrier" in lib.km_last_error(h)
    assert lib.km_set_wait_limit(h, -1) == L.KM_OK
    assert _assemble(lib, h, pts, *args) == L.KM_OK, lib.km_last_error(h)
    assert lib.km_factorize(h) == L.KM_OK, lib.km_last_error(h)
    x, ld = _solve_logdet(lib, h, rhs)
    fresh = _create(lib, L.KM_PREC_FP64)
    assert _assemble(lib, fresh, pts, *args) == L.KM_OK
    assert lib.km_factorize(fresh) == L.KM_OK
    x0, ld0 = _solve_logdet(lib, fresh, rhs)
    assert ld == ld0 and np.array_equal(x, x0)
    lib.km_destroy(h)
    lib.km_destroy(fresh)
