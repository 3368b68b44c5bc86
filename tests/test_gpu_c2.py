"""The benchmark workload itself (n = 2^16, Matern nu = 3/2, Nystrom rank 72, FixedLevel(8),
16 right-hand sides) against the oracle's fixture (tests/golden/make_c2_golden.py, the same
seeded inputs): logdet, 1024 sample rows and the column norms of the 16-column solve, and the
pre-factorisation matvec (baseoverloads.jl:152-209).  FP64 form: logdet within 1e-8 absolute,
solve within 1e-9 relative; mixed form: the stated targets, logdet within 1e-6 absolute and
solve within 1e-8 relative of the FP64 oracle.  The matvec is FP64 in both forms (1e-12)."""
import sys
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLD))
pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("mixed", [False, True])
def test_c2_workload_against_oracle(lib, mixed):
    import kmhodlr as K
    from make_c2_golden import inputs
    d = np.load(GOLD / "c2_n65536.npz")
    pts, rhs, xv, idx = inputs()
    assert np.array_equal(idx, d["idx"])
    prec = K.KM_PREC_MIXED if mixed else K.KM_PREC_FP64
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, d["params"], K.Matern32()), 0.0, int(d["rank"]),
                       K.FixedLevel(int(d["level"])), nystrom=True, precision=prec)
    y = hk @ xv
    K.symmetricfactorize(hk)
    x = hk.ldiv(rhs)
    ld = hk.logdet()
    assert rel(y[idx, 0], d["matvec_rows"]) < 1e-12
    assert abs(np.linalg.norm(y) - float(d["matvec_norm"])) / float(d["matvec_norm"]) < 1e-12
    ld_tol, x_tol = (1e-6, 1e-8) if mixed else (1e-8, 1e-9)
    assert abs(ld - float(d["logdet"])) < ld_tol
    assert rel(x[idx], d["solve_rows"]) < x_tol
    assert np.max(np.abs(np.linalg.norm(x, axis=0) / d["solve_colnorms"] - 1.0)) < x_tol
