"""The stochastic Hessian (km_stoch_hessian) against the oracle's restatement of stoch_hessian
(src/HODLR/src/stochastichessian.jl:117-147) on the same points, data and probes: both kernels,
FP64 and mixed forms, rel 1e-6 (FP64) / 1e-5 (mixed) of the largest entry, the tolerance of the
Fisher matrix it contains (the per-probe terms go through W^{-T}), and every entry to 1e-5 / 1e-4
of sqrt(|H_jj H_kk|).  The second-derivative terms
alone (Hessian + Fisher) are checked to the same bound, and the seeded form against the
explicit-probe form with the same probes."""
import numpy as np
import pytest

from oracle import hodlr_oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kid,params", [(O.KERNEL_MATERN32, (1.0, 0.1, 1e-2)), (O.KERNEL_RQ, (1.2, 0.15, 1e-2))])
@pytest.mark.parametrize("mixed", [False, True])
def test_stoch_hessian_matches_oracle(lib, kid, params, mixed):
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    n, rank, level = 2048, 32, 3
    pts = uniform_points(n, 43)
    y = np.random.default_rng(19).standard_normal(n)
    V = O.rademacher_probes(n, 8, 23)
    vecs = [V[:, c] for c in range(V.shape[1])]
    ok = O.KernelMatrix(pts, pts, np.array(params), kid)
    ohk = O.build_hodlr(ok, 0.0, rank, O.FixedLevel(level), nystrom=True)
    O.symmetricfactorize(ohk)
    H0 = O.stoch_hessian(ok, ohk, y, vecs)
    F0 = O.stoch_fisher(ok, ohk, [O.derivative_hodlr(ok, j, ohk) for j in range(3)], vecs)
    prec = K.KM_PREC_MIXED if mixed else K.KM_PREC_FP64
    kern = K.Matern32() if kid == O.KERNEL_MATERN32 else K.RatQuad()
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, params, kern), 0.0, rank, K.FixedLevel(level), nystrom=True,
                       precision=prec)
    K.symmetricfactorize(hk)
    nll, g, H = K.grad_fisher_hessian(hk, y, V)
    tol = (1e-5 if mixed else 1e-6) * np.max(np.abs(H0))
    # the entries span orders of magnitude: each is also checked against sqrt(|H_jj H_kk|)
    scale = np.sqrt(np.outer(np.abs(np.diag(H0)), np.abs(np.diag(H0))))
    etol = (1e-4 if mixed else 1e-5) * scale
    assert np.array_equal(H, H.T) and np.all(np.isfinite(H))
    assert np.max(np.abs(H - H0)) <= tol, (H, H0)
    assert np.all(np.abs(H - H0) <= etol), (H, H0)
    _, _, F = K.grad_and_fisher(hk, y, V)
    assert np.max(np.abs((H + F) - (H0 + F0))) <= tol
    assert np.all(np.abs((H + F) - (H0 + F0)) <= etol)
    nll2, g2, F2 = K.grad_and_fisher(hk, y, V)
    assert nll2 == nll and np.array_equal(g2, g)
    H2 = K.stoch_hessian(hk, y, nprobe=8, seed=23)
    assert np.array_equal(H2, H)
    if not mixed:  # the assemble + factorise + Hessian driver on a fresh FP64 handle
        assert np.array_equal(K.nll_hessian(params, pts, y, kern, rank, K.FixedLevel(level), V), H)


def test_hessian_after_reassembly_at_a_larger_shape(lib):
    """A handle that computed a Hessian at a small shape and is then reassembled at a larger one
    regrows its second-derivative workspace: the Hessian equals, bit for bit, that of a fresh
    handle at the larger shape."""
    import kmhodlr as K
    from kmhodlr import _lib as L
    from kmhodlr import hodlr as KH
    from kmhodlr.data import uniform_points
    params = np.array([1.0, 0.1, 1e-2])
    small = uniform_points(1024, 5)
    big = uniform_points(4096, 6)
    y_s = np.random.default_rng(1).standard_normal(1024)
    y_b = np.random.default_rng(2).standard_normal(4096)
    V_s = O.rademacher_probes(1024, 8, 3)
    V_b = O.rademacher_probes(4096, 8, 4)
    hk = K.KernelHODLR(K.KernelMatrix(small, small, params, K.Matern32()), 0.0, 16, K.FixedLevel(2),
                       nystrom=True)
    K.symmetricfactorize(hk)
    K.stoch_hessian(hk, y_s, V_s)
    kind, lv = KH._level(K.FixedLevel(4))
    pb = np.ascontiguousarray(big)
    rc = lib.km_assemble(hk._h, KH._dp(pb), 4096, int(K.Matern32().kid), KH._dp(params), 3,
                         L.KM_METHOD_NYSTROM, 0.0, 32, kind, lv)
    assert rc == L.KM_OK, lib.km_last_error(hk._h)
    hk.n = 4096
    K.symmetricfactorize(hk)
    H = K.stoch_hessian(hk, y_b, V_b)
    fresh = K.KernelHODLR(K.KernelMatrix(big, big, params, K.Matern32()), 0.0, 32, K.FixedLevel(4),
                          nystrom=True)
    K.symmetricfactorize(fresh)
    assert np.array_equal(H, K.stoch_hessian(fresh, y_b, V_b))


@pytest.mark.parametrize("kid,params", [(O.KERNEL_MATERN32, (1.0, 0.1, 1e-2)), (O.KERNEL_RQ, (1.2, 0.15, 1e-2))])
@pytest.mark.parametrize("mixed", [False, True])
def test_profile_hessian_matches_oracle(lib, kid, params, mixed):
    """km_stoch_profile_hessian against the oracle's stoch_hessian(..., profile = true)
    (HODLR_p_hess_slv, stochastichessian.jl:15-31) on the same points, data and probes, to the
    tolerances of the plain Hessian; its NLL and gradient are the profile likelihood's."""
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    n, rank, level = 2048, 32, 3
    pts = uniform_points(n, 47)
    y = np.random.default_rng(29).standard_normal(n)
    V = O.rademacher_probes(n, 8, 31)
    vecs = [V[:, c] for c in range(V.shape[1])]
    ok = O.KernelMatrix(pts, pts, np.array(params), kid)
    ohk = O.build_hodlr(ok, 0.0, rank, O.FixedLevel(level), nystrom=True)
    O.symmetricfactorize(ohk)
    H0 = O.stoch_hessian(ok, ohk, y, vecs, profile=True)
    nll0 = O.profile_negloglik(ohk, y)
    g0 = O.stoch_profile_gradient(ok, ohk, y, 3, vecs)
    prec = K.KM_PREC_MIXED if mixed else K.KM_PREC_FP64
    kern = K.Matern32() if kid == O.KERNEL_MATERN32 else K.RatQuad()
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, params, kern), 0.0, rank, K.FixedLevel(level), nystrom=True,
                       precision=prec)
    K.symmetricfactorize(hk)
    nll, g, H = K.grad_fisher_hessian(hk, y, V, profile=True)
    tol = (1e-5 if mixed else 1e-6) * np.max(np.abs(H0))
    scale = np.sqrt(np.outer(np.abs(np.diag(H0)), np.abs(np.diag(H0))))
    etol = (1e-4 if mixed else 1e-5) * scale
    assert np.array_equal(H, H.T) and np.all(np.isfinite(H))
    assert np.max(np.abs(H - H0)) <= tol, (H, H0)
    assert np.all(np.abs(H - H0) <= etol), (H, H0)
    assert abs(nll - nll0) <= (1e-9 if mixed else 1e-12) * abs(nll0)
    assert np.all(np.abs(g - g0) <= (1e-5 if mixed else 1e-6) * np.abs(g0) + 1e-8)
    # the profile form differs from the plain Hessian in its solve terms only
    assert not np.allclose(H, K.stoch_hessian(hk, y, V))
    assert np.array_equal(H, K.stoch_hessian(hk, y, V, profile=True))
