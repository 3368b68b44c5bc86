"""Host-side pieces of the batched and serving forms (no GPU): the device-bytes estimate that
drives admission, and the oracle twin of the engine's seeded Rademacher probes."""
import numpy as np

from oracle import hodlr_oracle as O


def test_estimate_bytes_shapes(lib):
    import kmhodlr as K
    lv = K.LogLevel(8)
    sizes = [1024, 2048, 4096, 8192, 32768]
    est = [K.estimate_bytes(n, 72, lv, 73, True) for n in sizes]
    assert all(e > 0 for e in est)
    assert all(a < b for a, b in zip(est, est[1:]))
    # the gradient workspaces and extra columns only add bytes
    assert K.estimate_bytes(4096, 72, lv, 1, False) < K.estimate_bytes(4096, 72, lv, 73, False) \
        < K.estimate_bytes(4096, 72, lv, 73, True)
    # the resident factor of an n-point problem holds at least its leaves twice (K and chol)
    n = 65536
    assert K.estimate_bytes(n, 72, K.FixedLevel(8), 1, False) > 2 * n * 256 * 8


def test_estimate_bytes_rejects_bad_shapes(lib):
    import kmhodlr as K
    assert K.estimate_bytes(0, 72, K.LogLevel(8)) == -1
    assert K.estimate_bytes(1024, 0, K.LogLevel(8)) == -1


def test_oracle_probe_twin():
    V = O.rademacher_probes(1000, 8, 123)
    assert V.shape == (1000, 8)
    assert set(np.unique(V)) == {-1.0, 1.0}
    assert abs(V.mean()) < 0.05
    assert np.array_equal(V, O.rademacher_probes(1000, 8, 123))
    assert not np.array_equal(V, O.rademacher_probes(1000, 8, 124))
    # column j of an n x p block is the same stream position whatever p is
    assert np.array_equal(O.rademacher_probes(1000, 3, 5), O.rademacher_probes(1000, 8, 5)[:, :3])
