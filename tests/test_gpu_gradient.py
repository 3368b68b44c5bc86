"""GPU parity of the derivative HODLR, the NLL and the stochastic gradient (rows a13-a15).

Tolerances: derivative products rel 1e-11 (same products, different summation order); NLL rel
1e-12; stochastic gradient rel 1e-6 against the oracle with the same probes (the per-probe trace
terms go through W^{-T}, which is fixed only to ~1e-9 relative, see test_gpu_nystrom.py)."""
import numpy as np
import pytest

from oracle import hodlr_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n,kid,params,rank,level", [
    (2048, O.KERNEL_MATERN32, (1.0, 0.1, 1e-3), 32, 3),
    (1500, O.KERNEL_RQ, (1.3, 0.2, 1e-2), 16, 2),
])
def test_derivative_nll_gradient(lib, n, kid, params, rank, level):
    import kmhodlr as K
    from kmhodlr.data import rademacher, uniform_points
    pts = uniform_points(n, n + 5)
    y = np.random.default_rng(n).standard_normal(n)
    V = rademacher(n, 24, n + 7)
    ok = O.KernelMatrix(pts, pts, np.array(params), kid)
    ohk = O.build_hodlr(ok, 0.0, rank, O.FixedLevel(level), nystrom=True)
    km = K.KernelMatrix(pts, pts, params, K.Matern32() if kid == 1 else K.RatQuad())
    hk = K.KernelHODLR(km, 0.0, rank, K.FixedLevel(level), nystrom=True)
    x = np.random.default_rng(1).standard_normal((n, 2))
    for j in range(3):
        DK = O.derivative_hodlr(ok, j, ohk)
        assert rel(hk.derivative_matvec(j, x), O.derivative_mul(DK, x)) < 1e-11
    O.symmetricfactorize(ohk)
    K.symmetricfactorize(hk)
    nll = K.negloglik(hk, y)
    assert abs(nll - O.negloglik(ohk, y)) < 1e-12 * abs(nll) + 1e-9
    g = K.stoch_gradient(hk, y, V)
    g0 = O.stoch_gradient(ok, ohk, y, 3, [V[:, c] for c in range(V.shape[1])])
    assert np.all(np.abs(g - g0) <= 1e-6 * np.abs(g0) + 1e-8)


def test_gradient_tracks_exact_hodlr_gradient(lib):
    import kmhodlr as K
    from kmhodlr.data import rademacher, uniform_points
    n, rank, level = 1024, 64, 2
    pts = uniform_points(n, 3)
    p = np.array([1.0, 0.1, 1e-3])
    y = np.random.default_rng(4).standard_normal(n)
    ok = O.KernelMatrix(pts, pts, p, O.KERNEL_MATERN32)
    g_exact = O.hodlr_exact_gradient(ok, rank, O.FixedLevel(level), y, 3)
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, p, K.Matern32()), 0.0, rank, K.FixedLevel(level), nystrom=True)
    K.symmetricfactorize(hk)
    g = K.stoch_gradient(hk, y, rademacher(n, 400, 9))
    assert np.all(np.abs(g - g_exact) < 0.05 * np.abs(g_exact) + 5.0)


def test_nll_objective_mirror(lib):
    import kmhodlr as K
    from kmhodlr.data import rademacher, uniform_points
    n = 2048
    pts = uniform_points(n, 8)
    y = np.random.default_rng(2).standard_normal(n)
    V = rademacher(n, 8, 3)
    grad = np.zeros(3)
    nll = K.nll_objective([1.0, 0.1, 1e-3], grad, pts, y, K.Matern32(), 32, K.FixedLevel(3), V)
    g0 = np.zeros(3)
    nll0 = O.nll_objective([1.0, 0.1, 1e-3], g0, pts, y, O.KERNEL_MATERN32, 32, O.FixedLevel(3),
                           [V[:, c] for c in range(8)])
    assert abs(nll - nll0) < 1e-10 * abs(nll0)
    assert np.all(np.abs(grad - g0) <= 1e-6 * np.abs(g0) + 1e-8)
