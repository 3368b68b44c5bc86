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


@pytest.mark.parametrize("mixed", [False, True])
def test_profile_likelihood_and_gradient(lib, mixed):
    """profile_negloglik / stoch_profile_gradient / nlpl_objective against the oracle with the
    same probes, in the FP64 form (NLL rel 1e-12, gradient rel 1e-6) and the mixed form (NLL abs
    1e-6 + rel 1e-9, gradient rel 1e-5)."""
    import kmhodlr as K
    from kmhodlr.data import rademacher, uniform_points
    n, rank, level = 2048, 32, 3
    pts = uniform_points(n, 12)
    p = (1.0, 0.1, 1e-3)
    y = np.random.default_rng(5).standard_normal(n)
    V = rademacher(n, 16, 6)
    vecs = [V[:, c] for c in range(V.shape[1])]
    ok = O.KernelMatrix(pts, pts, np.array(p), O.KERNEL_MATERN32)
    ohk = O.build_hodlr(ok, 0.0, rank, O.FixedLevel(level), nystrom=True)
    O.symmetricfactorize(ohk)
    prec = K.KM_PREC_MIXED if mixed else K.KM_PREC_FP64
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, p, K.Matern32()), 0.0, rank, K.FixedLevel(level), nystrom=True,
                       precision=prec)
    K.symmetricfactorize(hk)
    nll0 = O.profile_negloglik(ohk, y)
    g0 = O.stoch_profile_gradient(ok, ohk, y, 3, vecs)
    nll = K.profile_negloglik(hk, y)
    g = K.stoch_profile_gradient(hk, y, V)
    if mixed:
        assert abs(nll - nll0) < 1e-6 + 1e-9 * abs(nll0)
        assert np.all(np.abs(g - g0) <= 1e-5 * np.abs(g0) + 1e-6)
    else:
        assert abs(nll - nll0) < 1e-12 * abs(nll0)
        assert np.all(np.abs(g - g0) <= 1e-6 * np.abs(g0) + 1e-8)
        grad = np.zeros(3)
        assert K.nlpl_objective(p, grad, pts, y, K.Matern32(), rank, K.FixedLevel(level), V) == nll
        assert np.array_equal(grad, g)
        ya = float(y @ O.hodlr_ldiv(ohk, y))
        assert abs(K.scaleparm_mle(p, pts, y, K.Matern32(), rank, K.FixedLevel(level)) - ya / n) < 1e-12 * ya / n
    with pytest.raises(K.KMError, match="not positive"):
        K.profile_negloglik(hk, np.zeros(n))


def test_gpsimulate_is_factor_product(lib):
    """gpsimulate's HODLR branch (maxlikfunctions.jl:148-172) returns W z; W z has covariance
    W W' = the HODLR matrix, and equals the oracle's factor product to rel 1e-10."""
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    n, rank, level = 2048, 32, 3
    pts = uniform_points(n, 31)
    p = (1.0, 0.1, 1e-3)
    z = np.random.default_rng(8).standard_normal(n)
    out = K.gpsimulate(K.Matern32(), pts, p, rank, K.FixedLevel(level), z)
    ok = O.KernelMatrix(pts, pts, np.array(p), O.KERNEL_MATERN32)
    ohk = O.build_hodlr(ok, 0.0, rank, O.FixedLevel(level), nystrom=True)
    O.symmetricfactorize(ohk)
    assert rel(out, O.factor_mul(ohk.W, z)) < 1e-10


@pytest.mark.parametrize("mixed", [False, True])
def test_grad_and_fisher(lib, mixed):
    """km_grad_fisher against the oracle's stoch_fisher with the same probes (rel 1e-6 of the
    largest entry in FP64, 1e-5 mixed); its gradient equals km_nll_grad's bit for bit, and the
    seeded form equals the host-probe form with the same probes."""
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    n, rank, level = 2048, 32, 3
    pts = uniform_points(n, 41)
    p = (1.0, 0.1, 1e-3)
    y = np.random.default_rng(9).standard_normal(n)
    V = O.rademacher_probes(n, 12, 17)
    vecs = [V[:, c] for c in range(V.shape[1])]
    ok = O.KernelMatrix(pts, pts, np.array(p), O.KERNEL_MATERN32)
    ohk = O.build_hodlr(ok, 0.0, rank, O.FixedLevel(level), nystrom=True)
    O.symmetricfactorize(ohk)
    F0 = O.stoch_fisher(ok, ohk, [O.derivative_hodlr(ok, j, ohk) for j in range(3)], vecs)
    prec = K.KM_PREC_MIXED if mixed else K.KM_PREC_FP64
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, p, K.Matern32()), 0.0, rank, K.FixedLevel(level), nystrom=True,
                       precision=prec)
    K.symmetricfactorize(hk)
    nll, g, F = K.grad_and_fisher(hk, y, V)
    assert np.array_equal(F, F.T)
    assert np.max(np.abs(F - F0)) <= (1e-5 if mixed else 1e-6) * np.max(np.abs(F0))
    nll1, g1 = hk.nll_grad(y, V)
    # nll_grad sums x' dK x over the probes in trace form (leaf Gram matrices); grad_and_fisher
    # forms dK x column by column for the Fisher matrix: the same sum in another order
    assert nll == nll1 and np.allclose(g, g1, rtol=1e-10, atol=0.0)
    nll2, g2, F2 = K.grad_and_fisher(hk, y, nprobe=12, seed=17)
    assert nll2 == nll and np.array_equal(g2, g) and np.array_equal(F2, F)
    if not mixed:
        g3, F3 = K.grad_and_fisher_matrix(p, pts, y, K.Matern32(), rank, K.FixedLevel(level), V)
        assert np.array_equal(g3, g) and np.array_equal(F3, F)
