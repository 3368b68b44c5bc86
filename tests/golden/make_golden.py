"""Generates the golden fixtures of the parity tests from the CPU oracle.

Run from the repository root:  python tests/golden/make_golden.py
Every case records its seeds, inputs and the oracle's outputs (float64).  The oracle
(oracle/hodlr_oracle.py) restates the reference's algorithm; see its header for what pins it.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "kernelmatrices.jl_gb300"))

from oracle import hodlr_oracle as O  # noqa: E402
from kmhodlr.data import normal_points, uniform_points  # noqa: E402

OUT = Path(__file__).resolve().parent

NYSTROM_CASES = {
    # name: (n, seed, kernel id, params, rank, level kind, level, rhs columns)
    "nys_matern_2048": (2048, 11, O.KERNEL_MATERN32, (1.0, 0.1, 1e-3), 32, "fixed", 3, 4),
    "nys_rq_1500": (1500, 12, O.KERNEL_RQ, (1.3, 0.2, 1e-2), 16, "log", 7, 3),
    "nys_matern_4096_r72": (4096, 13, O.KERNEL_MATERN32, (1.0, 0.1, 1e-3), 72, "fixed", 4, 2),
}


def level(kind: str, lv: int):
    return O.FixedLevel(lv) if kind == "fixed" else O.LogLevel(lv)


def nystrom_case(name, n, seed, kid, params, rank, kind, lv, ncol):
    pts = uniform_points(n, seed)
    rng = np.random.default_rng(seed + 1000)
    rhs = rng.standard_normal((n, ncol))
    K = O.KernelMatrix(pts, pts, np.array(params), kid)
    HK = O.build_hodlr(K, 0.0, rank, level(kind, lv), nystrom=True)
    matvec = O.hodlr_mul(HK, rhs)
    O.symmetricfactorize(HK)
    out = dict(pts=pts, rhs=rhs, params=np.array(params), kid=kid, rank=rank,
               level_kind=0 if kind == "fixed" else 1, level=lv, seed=seed,
               matvec=matvec, logdet=O.hodlr_logdet(HK), solve=O.hodlr_ldiv(HK, rhs),
               factor_solve=O.factor_ldiv(HK.W, rhs), factor_solve_t=O.factor_ldiv_t(HK.W, rhs),
               landmarks=O.nystrom_landmarks(n, rank) + 1)
    np.savez_compressed(OUT / f"{name}.npz", **out)


def aca_case():
    # RQ p = [1, 1] plus 1.0 on the diagonal, N(0,1) points, ACA tol 1e-12, LogLevel(8)
    n, seed = 1024, 21
    pts = normal_points(n, seed)
    rhs = np.random.default_rng(seed + 1000).standard_normal((n, 1))
    K = O.KernelMatrix(pts, pts, np.array([1.0, 1.0, 1.0]), O.KERNEL_RQ)
    HK = O.build_hodlr(K, 1e-12, 0, O.LogLevel(8), nystrom=False)
    ranks = np.array([u.shape[1] for lv in HK.U for u in lv])
    piv_rows = [np.array(p[0]) for lv in HK.pivots for p in lv]
    piv_cols = [np.array(p[1]) for lv in HK.pivots for p in lv]
    matvec = O.hodlr_mul(HK, rhs)
    O.symmetricfactorize(HK)
    out = dict(pts=pts, rhs=rhs, params=np.array([1.0, 1.0, 1.0]), ranks=ranks, matvec=matvec,
               logdet=O.hodlr_logdet(HK), solve=O.hodlr_ldiv(HK, rhs),
               dense_logdet=np.linalg.slogdet(K.full())[1], dense_solve=np.linalg.solve(K.full(), rhs),
               seed=seed)
    for i, (r_, c_) in enumerate(zip(piv_rows, piv_cols)):
        out[f"piv_rows_{i}"] = r_
        out[f"piv_cols_{i}"] = c_
    np.savez_compressed(OUT / "aca_rq_1024.npz", **out)


def main():
    for name, args in NYSTROM_CASES.items():
        nystrom_case(name, *args)
        print("wrote", name)
    aca_case()
    print("wrote aca_rq_1024")


if __name__ == "__main__":
    main()
