"""GPU RKernelHODLR (km_rhodlr_*): the recursive product-only HODLR of K(x1, x2) for different
point sets and lengths (src/HODLR/src/constructor.jl:130-161).  On the rational-quadratic kernel
the ACA ranks and pivots of every block equal the oracle's exactly (the same ACA kernels as the
symmetric path); products agree with the oracle's recursive product to rel 1e-12 and with the
dense matrix to the ACA tolerance."""
import numpy as np
import pytest

from oracle import hodlr_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n1,n2,kid,params,tol,rank,lvl", [
    (1000, 700, O.KERNEL_RQ, (1.0, 0.2, 1e-2), 1e-10, 0, ("fixed", 3)),
    (513, 2048, O.KERNEL_RQ, (1.3, 0.1, 0.0), 1e-8, 0, ("log", 6)),
    (3000, 3000, O.KERNEL_MATERN32, (1.0, 0.1, 1e-3), 1e-8, 20, ("fixed", 4)),
    (16400, 16384, O.KERNEL_RQ, (1.0, 0.3, 1e-2), 1e-9, 0, ("fixed", 2)),
])
def test_rect_parity(lib, n1, n2, kid, params, tol, rank, lvl):
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    x1 = uniform_points(n1, n1 + 1)
    x2 = uniform_points(n2, n2 + 2)
    if n1 == n2:
        x2[::7] = x1[::7]  # shared points: the nugget term applies where x1 and x2 coincide
    olv = O.FixedLevel(lvl[1]) if lvl[0] == "fixed" else O.LogLevel(lvl[1])
    clv = K.FixedLevel(lvl[1]) if lvl[0] == "fixed" else K.LogLevel(lvl[1])
    ok = O.KernelMatrix(x1, x2, np.array(params), kid)
    oR = O.rkernel_hodlr(ok, tol, rank, olv)
    R = K.RKernelHODLR(K.KernelMatrix(x1, x2, params, K.Matern32() if kid == 1 else K.RatQuad()), tol, rank, clv)
    assert R.shape == O.rhodlr_shape(oR) == (n1, n2)
    blocks = O.rhodlr_blocks(oR)
    ranks = R.block_ranks()
    assert len(ranks) == len(blocks) == R.nblocks
    oranks = [b[0].shape[1] for b in blocks]
    if kid == O.KERNEL_RQ:
        assert list(ranks) == oranks
        for q, b in enumerate(blocks):
            rows, cols = R.aca_pivots(q)
            assert list(rows) == list(b[2]) and list(cols) == list(b[3])
    else:
        assert np.all(np.abs(np.array(ranks) - np.array(oranks)) <= 1)
    x = np.random.default_rng(3).standard_normal((n2, 3))
    y = R @ x
    assert y.shape == (n1, 3)
    y0 = np.column_stack([O.rhodlr_mul(oR, x[:, c]) for c in range(3)])
    assert rel(y, y0) < (1e-12 if kid == O.KERNEL_RQ else 1e-9)
    if n1 * n2 <= 4_000_000:
        assert rel(y, ok.full() @ x) < 1e3 * tol + 1e-12
    assert rel(R @ x[:, 0], y[:, 0]) < 1e-15


def test_rect_levels_and_errors(lib):
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    x1 = uniform_points(300, 1)
    x2 = uniform_points(100, 2)
    km = K.KernelMatrix(x1, x2, (1.0, 0.2, 0.0), K.RatQuad())
    R0 = K.RKernelHODLR(km, 1e-10, 0, K.FixedLevel(0))
    assert R0.nblocks == 0 and R0.nleaves == 1
    x = np.random.default_rng(1).standard_normal(100)
    ok = O.KernelMatrix(x1, x2, np.array([1.0, 0.2, 0.0]), O.KERNEL_RQ)
    assert rel(R0 @ x, ok.full() @ x) < 1e-14
    # LogLevel(5) on min size 100: floor(log2 100) - 5 = 1 level
    assert K.RKernelHODLR(km, 1e-10, 0, K.LogLevel(5)).levels == 1
    with pytest.raises(K.KMError, match="too many levels"):
        K.RKernelHODLR(km, 1e-10, 0, K.FixedLevel(8))
    with pytest.raises(K.KMError, match="negative depth"):
        K.RKernelHODLR(km, 1e-10, 0, K.LogLevel(9))
    with pytest.raises(K.KMError, match="symmetric matrices"):
        K.KernelHODLR(km, 1e-10, 0, K.LogLevel(5))
