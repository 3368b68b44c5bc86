"""km_factorize_solve (symmetricfactorize! then K \\ b in one call, the forward half of the solve
on a second stream behind the factorisation's dependency points) gives the same factor and the
same solution, bit for bit, as km_factorize followed by km_solve: FP64 and mixed forms, one and
many right-hand sides, a single-leaf tree, FP64 refinement of the mixed form, and an ACA handle
(which takes the two calls)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pair(n, rank, lvl, prec, seed, **kw):
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    pts = uniform_points(n, seed)
    km = K.KernelMatrix(pts, pts, (1.0, 0.1, 1e-3), K.Matern32())
    mk = lambda: K.KernelHODLR(km, 0.0, rank, lvl, nystrom=True, precision=prec, **kw)  # noqa: E731
    return mk(), mk()


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("n,rank,level,k", [(5000, 40, 4, 1), (16384, 72, 6, 16), (300, 20, 0, 3),
                                           (6000, 64, 5, 37)])
def test_fused_equals_two_calls(lib, prec, n, rank, level, k):
    import kmhodlr as K
    a, b = _pair(n, rank, K.FixedLevel(level), prec, 11 + n)
    rhs = np.random.default_rng(n + k).standard_normal((n, k))
    K.symmetricfactorize(a)
    x0 = a.ldiv(rhs)
    x1 = K.factorize_solve(b, rhs)
    assert np.array_equal(x0, x1)
    assert a.logdet() == b.logdet()
    x2 = rhs[:, :1].copy()
    assert np.array_equal(a.ldiv(x2), b.ldiv(x2))


def test_fused_with_refinement(lib):
    import kmhodlr as K
    a, b = _pair(8192, 72, K.FixedLevel(5), 1, 5, refine_max_iter=3)
    rhs = np.random.default_rng(3).standard_normal((8192, 4))
    K.symmetricfactorize(a)
    assert np.array_equal(a.ldiv(rhs), K.factorize_solve(b, rhs))


def test_fused_aca_handle(lib):
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    pts = uniform_points(4096, 8)
    km = K.KernelMatrix(pts, pts, (1.0, 0.1, 1e-2), K.Matern32())
    a = K.KernelHODLR(km, 1e-8, 0, K.LogLevel(8), nystrom=False)
    b = K.KernelHODLR(km, 1e-8, 0, K.LogLevel(8), nystrom=False)
    rhs = np.random.default_rng(4).standard_normal((4096, 2))
    K.symmetricfactorize(a)
    assert np.array_equal(a.ldiv(rhs), K.factorize_solve(b, rhs))
