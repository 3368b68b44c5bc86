"""GPU k-d ordering (km_kd_order, km_maxlikdata): the permutation must equal the oracle's bit for
bit (integer work), for random points, ties on a grid, duplicated points, signed zeros, every
leaf size from 1 up, and sizes that are not powers of two."""
import time

import numpy as np
import pytest

from oracle import hodlr_oracle as O

pytestmark = pytest.mark.gpu


def grid(nx, ny):
    return np.stack(np.meshgrid(np.arange(float(nx)), np.arange(float(ny))), -1).reshape(-1, 2)


@pytest.mark.parametrize("n,leaf", [(1, 32), (5, 1), (32, 32), (33, 32), (1000, 8), (4099, 1), (65537, 32)])
def test_random_points(lib, n, leaf):
    import kmhodlr as K
    P = np.random.default_rng(n + leaf).uniform(-1, 1, size=(n, 2))
    assert np.array_equal(K.kd_order(P, leaf), O.kd_order(P, leaf))


def test_ties_duplicates_signed_zero(lib):
    import kmhodlr as K
    g = grid(37, 29)
    cases = [g, np.concatenate([g, g[::5], g[::7]]), grid(300, 1),
             np.array([[0.0, 1.0], [-0.0, 1.0], [0.0, -0.0], [1.0, 0.0], [-0.0, -0.0]] * 97)]
    for P in cases:
        for leaf in (1, 4, 32):
            assert np.array_equal(K.kd_order(P, leaf), O.kd_order(P, leaf))


def test_maxlikdata(lib):
    import kmhodlr as K
    rng = np.random.default_rng(3)
    P = rng.uniform(size=(5000, 2))
    y = rng.standard_normal(5000)
    ps, ys = K.maxlikdata(P, y)
    perm = O.kd_order(P, 32)
    assert np.array_equal(ps, P[perm]) and np.array_equal(ys, y[perm])
    p0, y0 = K.maxlikdata(P, y, sortmethod=":Nothing")
    assert np.array_equal(p0, P) and np.array_equal(y0, y)
    with pytest.raises(K.KMError, match="The options are"):
        K.maxlikdata(P, y, sortmethod="hilbert")
    bad = P.copy()
    bad[7, 1] = np.nan
    with pytest.raises(K.KMError, match="not finite"):
        K.kd_order(bad)


def test_large(lib):
    """n = 2^18: the ordering equals the oracle's; its time is printed (input step, not timed by
    the C2 bench)."""
    import kmhodlr as K
    P = np.random.default_rng(18).uniform(size=(1 << 18, 2))
    t0 = time.perf_counter()
    perm = K.kd_order(P, 32)
    dt = time.perf_counter() - t0
    assert np.array_equal(perm, O.kd_order(P, 32))
    print(f"kd_order n=2^18: {dt * 1e3:.1f} ms including handle creation and copies")
