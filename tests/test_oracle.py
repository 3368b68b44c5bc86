"""The CPU oracle against what pins it: the reference's own test identities
(test/runtests.jl:28-45), the dense formulas of src/HODLR/src/exactmaxlik.jl, the Bessel form of
the Matern covariance, and the committed golden fixtures.  CPU only."""
from pathlib import Path

import numpy as np
import pytest
import scipy.linalg as sla

from oracle import hodlr_oracle as O

GOLD = Path(__file__).resolve().parent / "golden"


def kd(pts):
    from kmhodlr.data import kd_order
    return pts[kd_order(pts)]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def basic():
    """example/basicexample.jl-like fixture: points on [0,10]^2, k-d ordered, RQ kernel with a
    1e-12 nugget, Nystrom rank 72, LogLevel(8), tol eps (test/runtests.jl:15-22)."""
    rng = np.random.default_rng(2)
    pts = kd(rng.uniform(size=(1024, 2)) * 10.0)
    K = O.KernelMatrix(pts, pts, np.array([3.0, 0.5, 1e-12]), O.KERNEL_RQ)
    HK = O.build_hodlr(K, np.finfo(float).eps, 72, O.LogLevel(8), nystrom=True)
    HKf = O.hodlr_full(HK)
    O.symmetricfactorize(HK)
    return K, HK, HKf


def test_runtests_identities(basic):
    K, HK, HKf = basic
    W = O.factor_full(HK.W)
    tvec = np.random.default_rng(3).standard_normal(HKf.shape[0])
    assert np.allclose(W @ W.T, HKf, rtol=1.5e-8, atol=1e-12 * np.abs(HKf).max())     # :28
    assert np.isclose(np.linalg.slogdet(HKf)[1], O.hodlr_logdet(HK), rtol=1e-5)     # :31
    assert np.allclose(HKf @ tvec, O.hodlr_mul(HK, tvec), rtol=1.5e-8)               # :34
    assert rel(O.hodlr_ldiv(HK, tvec), np.linalg.solve(HKf, tvec)) < 1e-8             # :37
    t1 = O.factor_ldiv(HK.W, tvec)
    assert rel(t1, np.linalg.solve(W, tvec)) < 1e-8                                   # :40-41
    t2 = O.factor_ldiv_t(HK.W, t1)
    assert rel(t2, np.linalg.solve(W.T, t1)) < 1e-8                                   # :44-45


def test_aca_runtests_identities_and_dense():
    """C1-like ACA case: N(0,1) points, README RQ kernel p=[1,1] + 1.0 diagonal, tol 1e-12."""
    rng = np.random.default_rng(4)
    pts = rng.standard_normal((512, 2))
    K = O.KernelMatrix(pts, pts, np.array([1.0, 1.0, 1.0]), O.KERNEL_RQ)
    HK = O.build_hodlr(K, 1e-12, 0, O.LogLevel(7), nystrom=False)
    HKf = O.hodlr_full(HK)
    Kd = K.full()
    assert np.abs(HKf - Kd).max() < 1e-9 * np.abs(Kd).max()      # ACA at 1e-12 reproduces K
    O.symmetricfactorize(HK)
    b = rng.standard_normal(512)
    assert abs(O.hodlr_logdet(HK) - np.linalg.slogdet(Kd)[1]) < 1e-8
    assert rel(O.hodlr_ldiv(HK, b), np.linalg.solve(Kd, b)) < 1e-8


def test_aca_pivot_rules():
    # restrictedmaxabs: first strict maximum of |x| outside the excluded set (src/utils.jl:2-15)
    x = np.array([1.0, -3.0, 3.0, 2.0])
    assert O.restrictedmaxabs(x, set()) == (-3.0, 1)
    assert O.restrictedmaxabs(x, {1}) == (3.0, 2)
    assert O.restrictedmaxabs(np.zeros(3), {0}) == (0.0, 1)
    # a rank-1 matrix is recovered exactly with one pivot
    rng = np.random.default_rng(5)
    pts = rng.standard_normal((40, 2))
    K = O.KernelMatrix(pts[:20], pts[20:], np.array([1.0, 1e6, 0.0]), O.KERNEL_RQ)
    U, V, rows, cols = O.ACA(K, 1e-12, 0)
    assert np.allclose(U @ V.T, K.full(), rtol=1e-10)


def test_matern_closed_form_matches_bessel():
    x = np.concatenate([np.linspace(1e-7, 5, 400), [1e-9, 0.0, 20.0]])
    assert np.allclose(O.mtn_cor(1.5, x), O.mtn_cor_general(1.5, x), rtol=1e-13, atol=1e-300)


def test_matern_derivatives_by_finite_differences():
    rng = np.random.default_rng(6)
    a, b = rng.uniform(size=(5, 2)), rng.uniform(size=(7, 2))
    p = np.array([1.3, 0.2, 1e-3])
    for kid in (O.KERNEL_MATERN32, O.KERNEL_RQ):
        for j in range(2):
            h = 1e-6 * p[j]
            pp, pm = p.copy(), p.copy()
            pp[j] += h
            pm[j] -= h
            fd = (O.kernel_block(kid, a, b, pp) - O.kernel_block(kid, a, b, pm)) / (2 * h)
            assert np.allclose(O.dkernel_block(kid, j, a, b, p), fd, rtol=1e-6, atol=1e-9)


def test_nll_and_gradient_against_dense():
    rng = np.random.default_rng(7)
    n = 1024
    pts = kd(rng.uniform(size=(n, 2)))
    p = np.array([1.0, 0.1, 1e-3])
    K = O.KernelMatrix(pts, pts, p, O.KERNEL_MATERN32)
    y = rng.standard_normal(n)
    HK = O.build_hodlr(K, 0.0, 64, O.FixedLevel(2), nystrom=True)
    HKf = O.hodlr_full(HK)
    O.symmetricfactorize(HK)
    nll = O.negloglik(HK, y)
    F = sla.cho_factor(HKf)
    nll_dense_hodlr = np.sum(np.log(np.diag(F[0]))) + 0.5 * y @ sla.cho_solve(F, y)
    assert abs(nll - nll_dense_hodlr) < 1e-7 * abs(nll)
    # stochastic gradient with many probes approaches the exact gradient of the HODLR NLL
    g_exact = O.hodlr_exact_gradient(K, 64, O.FixedLevel(2), y, 3)
    vecs = O.givesaa(200, n, 11)
    g = O.stoch_gradient(K, HK, y, 3, vecs)
    assert np.all(np.abs(g - g_exact) < 0.05 * np.abs(g_exact) + 5.0)
    # the derivative matvec equals the dense derivative of the Nystrom HODLR
    for j in range(3):
        DK = O.derivative_hodlr(K, j, HK)
        assert np.allclose(O.derivative_mul(DK, y), O.derivative_full(DK) @ y, rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("case", ["nys_matern_2048", "nys_rq_1500"])
def test_golden_fixtures_reproduce(case):
    d = np.load(GOLD / f"{case}.npz")
    lvl = O.FixedLevel(int(d["level"])) if int(d["level_kind"]) == 0 else O.LogLevel(int(d["level"]))
    K = O.KernelMatrix(d["pts"], d["pts"], d["params"], int(d["kid"]))
    HK = O.build_hodlr(K, 0.0, int(d["rank"]), lvl, nystrom=True)
    assert rel(O.hodlr_mul(HK, d["rhs"]), d["matvec"]) < 1e-14
    O.symmetricfactorize(HK)
    assert abs(O.hodlr_logdet(HK) - float(d["logdet"])) < 1e-9
    assert rel(O.hodlr_ldiv(HK, d["rhs"]), d["solve"]) < 1e-12


def test_profile_likelihood_identities():
    """The profile NLL is the NLL minimised over a scale c of K (Nystrom HODLR(cK) = c HODLR(K)):
    profile = min_c nll(cK) + n/2 (log n - 1), attained at c = y'K^-1y / n (scaleparm_mle).
    The profile gradient differs from the NLL gradient (same probes) by 0.5 u_j (1 - n/q),
    u_j = y'K^-1 dK_j K^-1 y, q = y'K^-1 y (stochasticgradient.jl:14-26 vs :48-64)."""
    rng = np.random.default_rng(21)
    n = 768
    pts = kd(rng.uniform(size=(n, 2)))
    p = np.array([1.0, 0.1, 1e-3])
    y = rng.standard_normal(n)
    K = O.KernelMatrix(pts, pts, p, O.KERNEL_MATERN32)
    HK = O.build_hodlr(K, 0.0, 32, O.FixedLevel(2), nystrom=True)
    O.symmetricfactorize(HK)
    c = O.scaleparm_mle(HK, y)
    Kc = O.KernelMatrix(pts, pts, p * np.array([c, 1.0, c]), O.KERNEL_MATERN32)
    HKc = O.build_hodlr(Kc, 0.0, 32, O.FixedLevel(2), nystrom=True)
    O.symmetricfactorize(HKc)
    prof = O.profile_negloglik(HK, y)
    assert abs(prof - (O.negloglik(HKc, y) + 0.5 * n * (np.log(n) - 1.0))) < 1e-9 * abs(prof)
    for cc in (0.5 * c, 2.0 * c):
        Kx = O.KernelMatrix(pts, pts, p * np.array([cc, 1.0, cc]), O.KERNEL_MATERN32)
        HKx = O.build_hodlr(Kx, 0.0, 32, O.FixedLevel(2), nystrom=True)
        O.symmetricfactorize(HKx)
        assert O.negloglik(HKx, y) > O.negloglik(HKc, y)
    vecs = O.givesaa(6, n, 3)
    g = O.stoch_gradient(K, HK, y, 3, vecs)
    gp = O.stoch_profile_gradient(K, HK, y, 3, vecs)
    a = O.hodlr_ldiv(HK, y)
    q = float(y @ a)
    for j in range(3):
        u = float(a @ O.derivative_mul(O.derivative_hodlr(K, j, HK), a))
        assert abs(gp[j] - (g[j] + 0.5 * u * (1.0 - n / q))) < 1e-9 * (abs(gp[j]) + abs(u))


def test_stochastic_fisher():
    """stoch_fisher and grad_and_fisher_matrix agree (stochastichessian.jl:91-115,152-181); the
    Fisher matrix is symmetric positive semi-definite, its off-diagonal polarisation equals
    0.5 mean (A_j v)'(A_k v), and with many probes it approaches the exact HODLR Fisher matrix
    0.5 tr(HK^-1 dHK_j HK^-1 dHK_k)."""
    rng = np.random.default_rng(23)
    n, rank, lvl = 512, 32, O.FixedLevel(2)
    pts = kd(rng.uniform(size=(n, 2)))
    p = np.array([1.0, 0.1, 1e-3])
    y = rng.standard_normal(n)
    K = O.KernelMatrix(pts, pts, p, O.KERNEL_MATERN32)
    HK = O.build_hodlr(K, 0.0, rank, lvl, nystrom=True)
    O.symmetricfactorize(HK)
    DKs = [O.derivative_hodlr(K, j, HK) for j in range(3)]
    vecs = O.givesaa(8, n, 5)
    F = O.stoch_fisher(K, HK, DKs, vecs)
    g2, F2 = O.grad_and_fisher_matrix(p, pts, y, O.KERNEL_MATERN32, rank, lvl, vecs)
    assert np.allclose(F, F2, rtol=1e-12, atol=0)
    assert np.allclose(g2, O.stoch_gradient(K, HK, y, 3, vecs), rtol=1e-12, atol=1e-12)
    assert np.allclose(F, F.T) and np.all(np.linalg.eigvalsh(F) > -1e-9 * np.abs(F).max())
    A = [np.column_stack([O.factor_ldiv(HK.W, O.derivative_mul(D, O.factor_ldiv_t(HK.W, v))) for v in vecs])
         for D in DKs]
    for j in range(3):
        for k in range(3):
            assert abs(F[j, k] - 0.5 * np.mean(np.sum(A[j] * A[k], axis=0))) < 1e-10 * abs(F).max()
    HKf = O.hodlr_full(O.build_hodlr(K, 0.0, rank, lvl, nystrom=True))
    D = [O.derivative_full(DK) for DK in DKs]
    Si = np.linalg.inv(HKf)
    Fex = np.array([[0.5 * np.trace(Si @ D[j] @ Si @ D[k]) for k in range(3)] for j in range(3)])
    Fmc = O.stoch_fisher(K, HK, DKs, O.givesaa(300, n, 6))
    assert np.all(np.abs(Fmc - Fex) < 0.15 * np.sqrt(np.outer(np.diag(Fex), np.diag(Fex))))


def test_kd_order_oracle_matches_host_helper():
    """The oracle's recursive k-d ordering equals the host helper that generates the ordered test
    inputs (stack form of the same rule), also with ties, duplicates and signed zeros."""
    from kmhodlr.data import kd_order as host_kd
    rng = np.random.default_rng(5)
    g = np.stack(np.meshgrid(np.arange(23.0), np.arange(17.0)), -1).reshape(-1, 2)
    cases = [rng.uniform(size=(1000, 2)), g, np.concatenate([g, g[::3]]),
             np.array([[0.0, 1.0], [-0.0, 1.0], [0.0, -0.0], [1.0, 0.0]] * 20)]
    for P in cases:
        for leaf in (1, 7, 32):
            assert np.array_equal(O.kd_order(P, leaf), host_kd(P, leaf))


def test_second_derivatives_match_finite_differences():
    """d2kernel_block (the closed forms restated for the reference's user-supplied d2funs) is the
    parameter derivative of dkernel_block: central differences, both kernels, every pair."""
    rng = np.random.default_rng(11)
    x1, x2 = rng.uniform(size=(40, 2)), rng.uniform(size=(30, 2))
    x2[:5] = x1[:5]  # coincident points (the nugget indicator)
    for kid, p in ((O.KERNEL_MATERN32, [1.3, 0.2, 1e-2]), (O.KERNEL_RQ, [1.1, 0.15, 1e-2])):
        for j in range(3):
            for k in range(3):
                h = 1e-6 * max(abs(p[k]), 1e-3)
                pp, pm = list(p), list(p)
                pp[k] += h
                pm[k] -= h
                fd = (O.dkernel_block(kid, j, x1, x2, pp) - O.dkernel_block(kid, j, x1, x2, pm)) / (2 * h)
                d2 = O.d2kernel_block(kid, j, k, x1, x2, p)
                assert np.allclose(d2, fd, rtol=1e-6, atol=1e-7 * np.abs(fd).max() + 1e-12), (kid, j, k)
                assert np.array_equal(d2, O.d2kernel_block(kid, k, j, x1, x2, p))
                if O.d2_is_zero(kid, j, k):
                    assert not np.any(d2)


def sd_transforms(S, Sj, Sk, Sjk):
    """The reference's SDBlock_mul / SDBlock_mul_t as linear maps of the four projections
    [Phi' s; Phi_j' s; Phi_k' s; Phi_jk' s] to the four expansion coefficients (the form the GPU
    down-sweep applies): A = S^-1, B_x = A S_x A, C_jk = B_j S_k A, C_kj = B_k S_j A."""
    A = np.linalg.inv(S)
    Bj, Bk, Bjk = A @ Sj @ A, A @ Sk @ A, A @ Sjk @ A
    Cjk, Ckj = Bj @ Sk @ A, Bk @ Sj @ A
    Z = np.zeros_like(A)
    Tmul = np.block([[-Ckj + Bjk - Cjk - Bk, Bj, Z, A],
                     [-Bk, Z, A, Z],
                     [Bj + A, Z, Z, Z],
                     [A, Z, Z, Z]])
    Tmult = np.block([[-Cjk + Bjk - Ckj, -Bk, Bj, A],
                      [-Bk, Z, A, Z],
                      [Bj, Z, A, Z],
                      [A, Z, Z, Z]])
    return Tmul, Tmult


def test_sdblock_products_equal_their_projection_form():
    """SDBlock_mul and SDBlock_mul_t, restated term for term, equal the 4-projection transforms
    (rows: coefficients of Phi, Phi_j, Phi_k, Phi_jk) on random blocks."""
    rng = np.random.default_rng(12)
    r, mi, mj = 9, 31, 23
    G = rng.standard_normal((r, r))
    S = G @ G.T + r * np.eye(r)
    sym = lambda: (lambda M: M + M.T)(rng.standard_normal((r, r)))
    Sj, Sk, Sjk = sym(), sym(), sym()
    PhI = [rng.standard_normal((mi, r)) for _ in range(4)]   # Phi, Phi_j, Phi_k, Phi_jk on I
    PhJ = [rng.standard_normal((mj, r)) for _ in range(4)]   # the same on J
    Bj = O.DerivativeBlock(PhI[0], PhI[1], PhJ[0].T, PhJ[1].T)
    Bk = O.DerivativeBlock(PhI[0], PhI[2], PhJ[0].T, PhJ[2].T)
    Bjk = O.SecondDerivativeBlock(PhI[3], PhJ[3].T)
    Sc = sla.cho_factor(S, lower=False)
    Tmul, Tmult = sd_transforms(S, Sj, Sk, Sjk)
    sJ, sI = rng.standard_normal(mj), rng.standard_normal(mi)
    ref = O.sdblock_mul(Bj, Bk, Bjk, sJ, Sc, Sj, Sk, Sjk)
    c = Tmul @ np.concatenate([P.T @ sJ for P in PhJ])
    got = sum(PhI[v] @ c[v * r:(v + 1) * r] for v in range(4))
    assert np.allclose(got, ref, rtol=1e-10, atol=1e-10 * np.abs(ref).max())
    ref_t = O.sdblock_mul_t(Bj, Bk, Bjk, sI, Sc, Sj, Sk, Sjk)
    d = Tmult @ np.concatenate([P.T @ sI for P in PhI])
    got_t = sum(PhJ[v] @ d[v * r:(v + 1) * r] for v in range(4))
    assert np.allclose(got_t, ref_t, rtol=1e-10, atol=1e-10 * np.abs(ref_t).max())


def test_stoch_hessian_oracle():
    """stoch_hessian restated: symmetric, its no-second-derivative entries equal minus the Fisher
    entry minus half the solve term, and Deriv2mul is linear."""
    n, rank, lvl = 512, 24, O.FixedLevel(3)
    rng = np.random.default_rng(13)
    pts = rng.uniform(size=(n, 2))
    pts = pts[O.kd_order(pts, 16)]
    for kid, p in ((O.KERNEL_MATERN32, [1.0, 0.1, 1e-2]), (O.KERNEL_RQ, [1.0, 0.15, 1e-2])):
        K = O.KernelMatrix(pts, pts, np.asarray(p), kid)
        HK = O.build_hodlr(K, 0.0, rank, lvl, nystrom=True)
        O.symmetricfactorize(HK)
        y = rng.standard_normal(n)
        vecs = O.givesaa(6, n, 7)
        H = O.stoch_hessian(K, HK, y, vecs)
        assert np.array_equal(H, H.T) and np.all(np.isfinite(H))
        DKs = [O.derivative_hodlr(K, j, HK) for j in range(3)]
        F = O.stoch_fisher(K, HK, DKs, vecs)
        u = O.hodlr_ldiv(HK, y)
        assert abs(H[2, 2] - (-F[2, 2] - 0.5 * O.hess_slv_no2d(HK, DKs[2], DKs[2], y, u))) < 1e-10 * abs(H).max()
        D2B2, D2BL, Sjk = O.second_derivative_parts(K, HK, 0, 1)
        a, b = rng.standard_normal(n), rng.standard_normal(n)
        lhs = O.deriv2mul(DKs[0], DKs[1], D2B2, D2BL, Sjk, 2.0 * a - b)
        rhs = 2.0 * O.deriv2mul(DKs[0], DKs[1], D2B2, D2BL, Sjk, a) - O.deriv2mul(DKs[0], DKs[1], D2B2, D2BL, Sjk, b)
        assert np.allclose(lhs, rhs, rtol=1e-10, atol=1e-10 * np.abs(rhs).max())


def test_nystrom_landmark_identity():
    """Every off-diagonal block of a Nystrom HODLR is Phi_I S^-1 Phi_J' with the one landmark set
    (nystrom_uvt, src/factorizations.jl:86-94), and every derivative block is
    Phi_j,I S^-1 Phi_J' - Phi_I S^-1 S_j S^-1 Phi_J' + Phi_I S^-1 Phi_j,J' (DBlock_mul,
    src/HODLR/src/utils.jl:76-82).  The blocks on a leaf's path to the root hold every other leaf
    once, so with the leaf projections p_l = Phi_l' x_l, q_l = Phi_j,l' x_l and their sums P, Q:

    * K x on leaf i = L_i x_i + Phi_i S^-1 (P - p_i), the sibling sums as total minus own leaf;
    * dK x on leaf i = dL_i x_i + Phi_j,i S^-1 (P - p_i) - Phi_i S^-1 S_j S^-1 (P - p_i)
      + Phi_i S^-1 (Q - q_i);
    * x' dK x = sum_i x_i' dL_i x_i + f(P, Q) - sum_i f(p_i, q_i), f(p, q) = 2 u'q - u' S_j u with
      u = S^-1 p (the quadratic form of the trace-form gradient).

    Checked against the restated block-by-block products (baseoverloads.jl:152-179, 216-234)."""
    n, rank = 768, 20
    rng = np.random.default_rng(14)
    pts = rng.uniform(size=(n, 2))
    pts = pts[O.kd_order(pts, 16)]
    for kid, p in ((O.KERNEL_MATERN32, [1.2, 0.1, 1e-2]), (O.KERNEL_RQ, [0.9, 0.15, 1e-2])):
        K = O.KernelMatrix(pts, pts, np.asarray(p), kid)
        HK = O.build_hodlr(K, 0.0, rank, O.FixedLevel(4), nystrom=True)
        lnd = pts[O.nystrom_landmarks(n, rank)]
        Sc = sla.cho_factor(O.kernel_block(kid, lnd, lnd, p), lower=False)
        x = rng.standard_normal((n, 3))
        leaves = [(a - 1, b) for a, b, _, _ in HK.leafindices]
        phi = [O.kernel_block(kid, pts[a:b], lnd, p) for a, b in leaves]
        P_l = [f.T @ x[a:b] for f, (a, b) in zip(phi, leaves)]
        P = sum(P_l)
        got = np.concatenate([HK.L[i] @ x[a:b] + phi[i] @ sla.cho_solve(Sc, P - P_l[i])
                              for i, (a, b) in enumerate(leaves)])
        ref = O.hodlr_mul(HK, x)
        assert rel(got, ref) < 1e-12
        for j in range(3):
            DK = O.derivative_hodlr(K, j, HK)
            Sj = O.dkernel_block(kid, j, lnd, lnd, p)
            phj = [O.dkernel_block(kid, j, pts[a:b], lnd, p) for a, b in leaves]
            Q_l = [f.T @ x[a:b] for f, (a, b) in zip(phj, leaves)]
            Q = sum(Q_l)
            got = []
            for i, (a, b) in enumerate(leaves):
                u = sla.cho_solve(Sc, P - P_l[i])
                got.append(DK.L[i] @ x[a:b] + phj[i] @ u - phi[i] @ sla.cho_solve(Sc, Sj @ u)
                           + phi[i] @ sla.cho_solve(Sc, Q - Q_l[i]))
            ref = O.derivative_mul(DK, x)
            assert rel(np.concatenate(got), ref) < 1e-11

            def f(pp, qq):
                u = sla.cho_solve(Sc, pp)
                return np.einsum("rc,rc->c", u, 2.0 * qq - Sj @ u)

            quad = sum(np.einsum("rc,rc->c", x[a:b], DK.L[i] @ x[a:b]) for i, (a, b) in enumerate(leaves))
            quad = quad + f(P, Q) - sum(f(P_l[i], Q_l[i]) for i in range(len(leaves)))
            qref = np.einsum("rc,rc->c", x, ref)
            assert np.allclose(quad, qref, rtol=1e-10, atol=1e-10 * np.abs(qref).max())
