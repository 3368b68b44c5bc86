"""GPU tests of the batched (C4) and serving (C5) forms.

* seeded device probes equal the oracle twin: the NLL/gradient with device-drawn probes equals,
  bit for bit, the one with the same probes copied from the host;
* every problem of a concurrent batch equals, bit for bit, the same problem run alone on one
  handle, and matches the oracle (NLL rel 1e-12, gradient rel 1e-6 as in test_gpu_gradient.py);
* a request gives the same result alone and in a mix of concurrent requests (bit for bit);
* admission: a request whose estimate exceeds the HBM budget is rejected with KM_ERR_OOM while
  the others complete, and the server never reserves more than its budget."""
import numpy as np
import pytest

from oracle import hodlr_oracle as O

pytestmark = pytest.mark.gpu

RANK = 72


def problems(sizes, seed=0):
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    out = []
    for b, n in enumerate(sizes):
        pts = uniform_points(n, seed + 11 * b + 1)
        rho = float(np.exp(np.random.default_rng(seed + b).uniform(np.log(0.02), np.log(0.3))))
        y = np.random.default_rng(seed + 100 + b).standard_normal(n)
        out.append(K.Problem(pts, y, (1.0, rho, 1e-3)))
    return out


def single(prob, nprobe, seed, lvl, precision=0):
    import kmhodlr as K
    hk = K.KernelHODLR(K.KernelMatrix(prob.pts, prob.pts, prob.params, K.Matern32()), 0.0, RANK, lvl,
                       nystrom=True, precision=precision)
    K.symmetricfactorize(hk)
    return hk, hk.nll_grad_seeded(prob.y, nprobe, seed)


def test_seeded_probes_equal_host_probes(lib):
    import kmhodlr as K
    (prob,) = problems([2048], seed=3)
    hk, (nll_s, g_s) = single(prob, 16, 77, K.LogLevel(8))
    nll_h, g_h = hk.nll_grad(prob.y, O.rademacher_probes(2048, 16, 77))
    assert nll_s == nll_h
    assert np.array_equal(g_s, g_h)
    # the admission estimate bounds what the handle really holds
    assert hk.stats().device_bytes <= K.estimate_bytes(2048, RANK, K.LogLevel(8), 17, True)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_batch_equals_single_and_oracle(lib, precision):
    """Both forms: the batch equals single handles of the same form bit for bit; the oracle
    tolerances are those of the FP64 form (NLL rel 1e-12, gradient 1e-6) and, for the mixed form,
    its stated targets carried to the NLL (rel 1e-9) and gradient (rel 1e-5)."""
    import kmhodlr as K
    lvl = K.LogLevel(8)
    probs = problems([1024, 3000, 1500, 4096, 2048, 1200], seed=5)
    eng = K.BatchEngine(nworkers=3, precision=precision)
    nll, grad, status = eng.nll_grad(probs, K.Matern32(), RANK, lvl, nprobe=72, seed=1000)
    assert np.all(status == 0)
    for b, p in enumerate(probs):
        _, (nll1, g1) = single(p, 72, 1000 + b, lvl, precision)
        assert nll[b] == nll1, b
        assert np.array_equal(grad[b], g1), b
    # oracle parity on two of them with 8 probes
    nll8, grad8, _ = eng.nll_grad(probs[:2], K.Matern32(), RANK, lvl, nprobe=8, seed=50)
    for b in range(2):
        p = probs[b]
        n = len(p.y)
        ok = O.KernelMatrix(p.pts, p.pts, np.array(p.params), O.KERNEL_MATERN32)
        ohk = O.build_hodlr(ok, 0.0, RANK, O.LogLevel(8), nystrom=True)
        O.symmetricfactorize(ohk)
        nll_tol, g_tol = (1e-12, 1e-6) if precision == 0 else (1e-9, 1e-5)
        assert abs(nll8[b] - O.negloglik(ohk, p.y)) < nll_tol * abs(nll8[b]) + 1e-9
        V = O.rademacher_probes(n, 8, 50 + b)
        g0 = O.stoch_gradient(ok, ohk, p.y, 3, [V[:, c] for c in range(8)])
        assert np.all(np.abs(grad8[b] - g0) <= g_tol * np.abs(g0) + 1e-8)
    eng.close()


def test_profile_batch_and_serve_equal_single(lib):
    """The profile form (nlpl_objective, maxlikfunctions.jl:61-82) through the batch and the
    server equals a single handle bit for bit, in a mix with ordinary likelihood requests."""
    import kmhodlr as K
    lvl = K.LogLevel(8)
    probs = problems([2048, 1024, 3000, 1500], seed=31)
    eng = K.BatchEngine(nworkers=2)
    nll, grad, status = eng.nll_grad(probs, K.Matern32(), RANK, lvl, nprobe=16, seed=400, profile=True)
    assert np.all(status == 0)
    ones = []
    for b, p in enumerate(probs):
        hk, _ = single(p, 0, 0, lvl)
        ones.append(hk.nll_grad_seeded(p.y, 16, 400 + b, profile=True))
        assert nll[b] == ones[b][0], b
        assert np.array_equal(grad[b], ones[b][1]), b
    eng.close()
    srv = K.Server(K.Matern32(), RANK, lvl, nworkers=3)
    tp = [srv.submit_nll_grad(p, nprobe=16, seed=400 + b, profile=True) for b, p in enumerate(probs)]
    tn = [srv.submit_nll_grad(p, nprobe=16, seed=400 + b) for b, p in enumerate(probs)]
    for b in range(len(probs)):
        r = srv.wait(tp[b])
        assert r.status == 0 and r.nll == ones[b][0] and np.array_equal(r.grad, ones[b][1])
        assert srv.wait(tn[b]).nll != r.nll
    srv.close()


def test_batch_reports_failing_problem_and_continues(lib):
    import kmhodlr as K
    probs = problems([2048, 1500, 1024], seed=9)
    probs[1].params = (1.0, -0.1, 1e-3)  # a negative range is rejected by the assembly
    eng = K.BatchEngine(nworkers=2)
    nll, grad, status = eng.nll_grad(probs, K.Matern32(), RANK, K.LogLevel(8), nprobe=4, seed=1,
                                     raise_on_error=False)
    assert status[1] == 1  # KM_ERR_BAD_ARG
    assert status[0] == 0 and status[2] == 0
    assert np.isfinite(nll[0]) and np.isfinite(nll[2])
    with pytest.raises(K.KMError):
        eng.nll_grad(probs, K.Matern32(), RANK, K.LogLevel(8), nprobe=4, seed=1)
    eng.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_serve_same_alone_and_in_mix(lib, precision):
    import kmhodlr as K
    lvl = K.LogLevel(8)
    probs = problems([2048, 1024, 4096, 1500, 3000, 1024, 2048, 8192], seed=21)
    srv = K.Server(K.Matern32(), RANK, lvl, nworkers=4, precision=precision)
    alone = srv.wait(srv.submit_nll_grad(probs[0], nprobe=72, seed=9))
    assert alone.status == 0
    fa = srv.wait(srv.submit_factor(probs[2]))
    assert fa.status == 0 and fa.factor_id > 0
    rhs = np.random.default_rng(2).standard_normal((4096, 3))
    x_alone = srv.wait(srv.submit_solve(fa.factor_id, rhs)).x
    # the mix: likelihoods, another factor, solves on the first factor, all in flight together
    tickets = [srv.submit_nll_grad(p, nprobe=72, seed=100 + i) for i, p in enumerate(probs[1:])]
    t_again = srv.submit_nll_grad(probs[0], nprobe=72, seed=9)
    t_fac = srv.submit_factor(probs[3])
    t_solves = [srv.submit_solve(fa.factor_id, rhs) for _ in range(3)]
    mixed = srv.wait(t_again)
    assert mixed.status == 0
    assert mixed.nll == alone.nll and np.array_equal(mixed.grad, alone.grad)
    for t in t_solves:
        r = srv.wait(t)
        assert r.status == 0 and np.array_equal(r.x, x_alone)
    for t in tickets:
        assert srv.wait(t).status == 0
    fb = srv.wait(t_fac)
    assert fb.status == 0
    # the factor's logdet and solve equal a single handle's
    hk, _ = single(probs[2], 0, 0, lvl, precision)
    assert fa.logdet == hk.logdet()
    assert np.array_equal(x_alone, hk.ldiv(rhs))
    assert srv.wait(srv.submit_release(fa.factor_id)).status == 0
    assert srv.wait(srv.submit_solve(fa.factor_id, rhs)).status == 1  # released: KM_ERR_BAD_ARG
    st = srv.stats()
    assert st.completed >= 14 and st.failed == 1 and st.rejected == 0
    assert st.resident_factors == 1
    assert 0 < st.p50_ms <= st.p99_ms
    srv.close()


def test_serve_budget_admission(lib):
    import kmhodlr as K
    lvl = K.LogLevel(8)
    big = K.estimate_bytes(8192, RANK, lvl, 73, True)
    small = K.estimate_bytes(1024, RANK, lvl, 73, True)
    import torch
    total = torch.cuda.get_device_properties(0).total_memory
    frac = (3 * small) / total  # room for about three small requests, not for the big one
    assert 3 * small < big
    srv = K.Server(K.Matern32(), RANK, lvl, nworkers=4, hbm_budget_fraction=frac)
    probs = problems([1024] * 6, seed=31) + problems([8192], seed=41)
    ts = [srv.submit_nll_grad(p, nprobe=72, seed=i) for i, p in enumerate(probs)]
    res = [srv.wait(t) for t in ts]
    assert all(r.status == 0 for r in res[:6])
    assert res[6].status == 3  # KM_ERR_OOM
    st = srv.stats()
    assert st.rejected == 1 and st.completed == 6
    assert st.peak_bytes <= st.budget_bytes
    srv.close()
