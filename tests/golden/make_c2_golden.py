"""Generates the n = 2^16 parity fixture (tests/golden/c2_n65536.npz) from the CPU oracle.

Run from the repository root:  python tests/golden/make_c2_golden.py
The inputs are those of the benchmark workload, regenerated by the test from the same seeds:
65536 points uniform on [0, 1]^2 from default_rng(20260101), k-d ordered; Matern nu = 3/2
(variance 1, range 0.1) plus a 1e-3 nugget; Nystrom rank 72; FixedLevel(8); 16 N(0, 1)
right-hand sides and one matvec vector from default_rng(20260201).  The oracle
(oracle/hodlr_oracle.py, the reference's algorithm with its plel maps on a thread pool) gives
logdet, the solve and the pre-factorisation matvec; the fixture keeps logdet, the column norms
and 1024 seeded sample rows of the solve and of the matvec (the full arrays would be 8 MB).
"""
from __future__ import annotations

import os
import sys
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "kernelmatrices.jl_gb300"))

from oracle import hodlr_oracle as O  # noqa: E402
from kmhodlr.data import uniform_points  # noqa: E402

OUT = Path(__file__).resolve().parent / "c2_n65536.npz"
N, RANK, LEVEL, NRHS = 65536, 72, 8, 16
PARAMS = (1.0, 0.1, 1e-3)
PTS_SEED, RHS_SEED, IDX_SEED = 20260101, 20260201, 20260301
NSAMPLE = 1024


def inputs():
    pts = uniform_points(N, PTS_SEED)
    rng = np.random.default_rng(RHS_SEED)
    rhs = rng.standard_normal((N, NRHS))
    xv = rng.standard_normal((N, 1))
    idx = np.sort(np.random.default_rng(IDX_SEED).choice(N, size=NSAMPLE, replace=False))
    return pts, rhs, xv, idx


def main():
    if os.environ.get("OPENBLAS_NUM_THREADS") != "1":
        os.environ["OPENBLAS_NUM_THREADS"] = "1"
        os.execv(sys.executable, [sys.executable, *sys.argv])
    pts, rhs, xv, idx = inputs()
    pool = ThreadPoolExecutor(os.cpu_count() or 1)
    t0 = time.perf_counter()
    K = O.KernelMatrix(pts, pts, np.array(PARAMS), O.KERNEL_MATERN32)
    HK = O.build_hodlr(K, 0.0, RANK, O.FixedLevel(LEVEL), nystrom=True, pool=pool)
    y = O.hodlr_mul(HK, xv)
    O.symmetricfactorize(HK, pool=pool)
    x = O.hodlr_ldiv(HK, rhs)
    ld = O.hodlr_logdet(HK)
    np.savez_compressed(OUT, n=N, rank=RANK, level=LEVEL, params=np.array(PARAMS), pts_seed=PTS_SEED,
                        rhs_seed=RHS_SEED, idx=idx, logdet=ld, solve_rows=x[idx],
                        solve_colnorms=np.linalg.norm(x, axis=0), matvec_rows=y[idx, 0],
                        matvec_norm=np.linalg.norm(y))
    print(f"{OUT.name}: logdet {ld!r} ({time.perf_counter() - t0:.1f} s)")


if __name__ == "__main__":
    main()
