"""CPU oracle: a line-faithful NumPy/SciPy FP64 restatement of the KernelMatrices.jl HODLR hot path.

TEST INFRASTRUCTURE ONLY.  This module is the checker for the CUDA engine.  Only the test suite,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may
import it.  The product path (the C-ABI library and its Python/Julia mirrors) never calls it.

Every function names the reference file:line it restates (paths inside the KernelMatrices.jl
project).  The reference is pure Julia; Julia is not installed where this project is built, so no
output of the reference itself exists here.  What pins this restatement:

* the reference's own test identities (``test/runtests.jl:28-45``: W*W' == full(HK), logdet,
  matvec, solve, factor solve, factor-transpose solve), re-run on this oracle in ``tests/``;
* the reference's dense formulas (``src/HODLR/src/exactmaxlik.jl:2-17,42-48,62-69``), restated in
  ``dense_*`` below and compared against the HODLR results in ``tests/``;
* hand-derived known answers for the integer tree partition (``src/HODLR/src/indices.jl``).

No numeric golden vector produced by the Julia reference exists, so element-level parity with the
Julia program itself is **parity unpinned**; the golden fixtures under ``tests/golden/`` are
produced by this oracle (script committed beside them) and pin the CUDA engine to it.

Third-party arithmetic restated here: SpecialFunctions 2.0.0 / OpenSpecFun_jll 0.5.5+0 ``besselk``
(Manifest.toml:298-302, 235-239) is replaced by ``scipy.special.kv`` for general nu and by the
exact closed form at nu = 3/2; LAPACK (OpenBLAS) ``cholesky``/``qr!``/triangular ``ldiv!`` by
NumPy/SciPy LAPACK calls of the same algorithms.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence, Tuple

import numpy as np
import scipy.linalg as sla
import scipy.special as sps

# ----------------------------------------------------------------------------------------------
# Tree partition: src/HODLR/src/indices.jl, level types src/HODLR/src/structstypes.jl:30-37
# ----------------------------------------------------------------------------------------------


@dataclass(frozen=True)
class FixedLevel:
    """``FixedLevel(lv)`` (src/HODLR/src/structstypes.jl:30-32)."""
    lv: int


@dataclass(frozen=True)
class LogLevel:
    """``LogLevel(lv)``: depth floor(log2 n) - lv (src/HODLR/src/structstypes.jl:35-37)."""
    lv: int


def _floor_log2(N: int) -> int:
    """``Int64(floor(log2(N)))`` for 1 <= N < 2^48, where the Float64 log2 cannot round up."""
    if N < 1 or N >= (1 << 48):
        raise ValueError("N must satisfy 1 <= N < 2^48")
    return N.bit_length() - 1


def leafsizes(N: int, lvl) -> Tuple[int, List[int]]:
    """``_leafsizes`` (src/HODLR/src/indices.jl:5-24)."""
    fl = _floor_log2(N)
    if isinstance(lvl, FixedLevel):
        n = min(max(0, lvl.lv), fl)
    else:
        if lvl.lv < 0:
            raise ValueError("Please provide a positive value for the level offset.")
        n = min(max(0, fl - lvl.lv), fl)
    szs = [N // (2 ** n)] * (2 ** n)
    rem = N - sum(szs)
    while rem > 0:
        for j in range(len(szs)):
            szs[j] += 1
            rem -= 1
            if rem == 0:
                break
    return n, szs


def leafindices(szs: Sequence[int]) -> List[Tuple[int, int, int, int]]:
    """``_leafindices`` (indices.jl:29-37): 1-based inclusive [s, e, s, e] per leaf."""
    out = []
    strt = 1
    for s in szs:
        out.append((strt, strt + s - 1, strt, strt + s - 1))
        strt += s
    return out


def nextlevel(lf: Sequence[Tuple[int, int, int, int]], lvl: int) -> List[Tuple[int, int, int, int]]:
    """``_nextlevel`` (indices.jl:40-51): rows a:b = second child, cols c:d = first child."""
    out = []
    skp = 2 ** lvl
    skpd2 = 2 ** (lvl - 1)
    j = 1
    while j <= len(lf) - 1:
        out.append((lf[j + skpd2 - 1][0], lf[j + skp - 2][1], lf[j - 1][2], lf[j + skpd2 - 2][3]))
        j += skp
    return out


def HODLRindices(N: int, lvl):
    """``HODLRindices`` (indices.jl:55-65).  Returns (levels, leaf indices, non-leaf indices).

    As in the reference, the non-leaf list always holds at least one (possibly empty) level."""
    lv, szs = leafsizes(N, lvl)
    lfind = leafindices(szs)
    nonlf = [nextlevel(lfind, 1)]
    for j in range(2, lv + 1):
        nonlf.append(nextlevel(lfind, j))
    return lv, lfind, nonlf


# ----------------------------------------------------------------------------------------------
# Covariance functions: src/covariancefunctions.jl, README.md:42-48
# ----------------------------------------------------------------------------------------------

KERNEL_RQ = 0        # README.md:42-48 kernelfunction: p1^2/(1+(r/p2)^2)^2, plus nugget on x == y
KERNEL_MATERN32 = 1  # mtn_kernfun (covariancefunctions.jl:258-266) at nu = 3/2, plus nugget on x == y
SQRT3 = math.sqrt(3.0)


def _pairwise(x1: np.ndarray, x2: np.ndarray):
    dx = x1[:, None, 0] - x2[None, :, 0]
    dy = x1[:, None, 1] - x2[None, :, 1]
    r = np.sqrt(dx * dx + dy * dy)
    same = (x1[:, None, 0] == x2[None, :, 0]) & (x1[:, None, 1] == x2[None, :, 1])
    return r, same


def mtn_cor(nu: float, x: np.ndarray) -> np.ndarray:
    """``mtn_cor`` (covariancefunctions.jl:209-212) = p1*p2*p3 (:152-189), 1 when |x| <= 1e-8."""
    x = np.asarray(x, dtype=np.float64)
    out = np.ones_like(x)
    m = np.abs(x) > 1.0e-8
    xm = x[m]
    if nu == 1.5:
        z = SQRT3 * xm
        out[m] = (1.0 + z) * np.exp(-z)
    else:
        z = math.sqrt(2.0 * nu) * xm
        out[m] = (z ** nu) * sps.kv(nu, z) / (math.gamma(nu) * 2.0 ** (nu - 1.0))
    return out


def mtn_cor_general(nu: float, x: np.ndarray) -> np.ndarray:
    """``mtn_cor`` through the Bessel function for any nu (used to pin the nu = 3/2 closed form)."""
    x = np.asarray(x, dtype=np.float64)
    out = np.ones_like(x)
    m = np.abs(x) > 1.0e-8
    z = math.sqrt(2.0 * nu) * x[m]
    out[m] = (z ** nu) * sps.kv(nu, z) / (math.gamma(nu) * 2.0 ** (nu - 1.0))
    return out


def mtn_cor_dx(nu: float, x: np.ndarray) -> np.ndarray:
    """``mtn_cor_dx`` (covariancefunctions.jl:214-217); nu = 3/2: d/dx (1+sqrt3 x)e^{-sqrt3 x}."""
    if nu != 1.5:
        raise NotImplementedError("only nu = 3/2 is on the path")
    x = np.asarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    m = np.abs(x) > 1.0e-8
    xm = x[m]
    out[m] = -3.0 * xm * np.exp(-SQRT3 * xm)
    return out


def kernel_block(kid: int, x1: np.ndarray, x2: np.ndarray, p: Sequence[float]) -> np.ndarray:
    """Dense block [k(x, y, p) for x in x1, y in x2] (src/baseoverloads.jl:10-12)."""
    r, same = _pairwise(x1, x2)
    if kid == KERNEL_RQ:
        # README.md:42-48 (out = abs2(p1)/abs2(1 + abs2(r/p2)); x == y adds the nugget)
        out = (p[0] * p[0]) / np.square(1.0 + np.square(r / p[1]))
    elif kid == KERNEL_MATERN32:
        # mtn_kernfun (covariancefunctions.jl:258-266): t0 * mtn_cor(nu, r/t1) when r > 0
        out = np.full(r.shape, float(p[0]))
        pos = r > 0.0
        out[pos] = p[0] * mtn_cor(1.5, r[pos] / p[1])
    else:
        raise ValueError("unknown kernel id")
    return out + np.where(same, float(p[2]), 0.0)


def dkernel_block(kid: int, j: int, x1: np.ndarray, x2: np.ndarray, p: Sequence[float]) -> np.ndarray:
    """Derivative of ``kernel_block`` in parameter j (0: scale, 1: range, 2: nugget).

    Matern: ``mtn_kernfun_d1`` (covariancefunctions.jl:268-276), ``mtn_kernfun_d2`` (:278-286);
    the nugget derivative is the indicator x == y."""
    r, same = _pairwise(x1, x2)
    if j == 2:
        return np.where(same, 1.0, 0.0)
    if kid == KERNEL_RQ:
        u = 1.0 + np.square(r / p[1])
        if j == 0:
            return 2.0 * p[0] / np.square(u)
        return 4.0 * p[0] * p[0] * np.square(r) / (p[1] ** 3) / (u * u * u)
    if kid == KERNEL_MATERN32:
        pos = r > 0.0
        if j == 0:
            out = np.ones(r.shape)
            out[pos] = mtn_cor(1.5, r[pos] / p[1])
            return out
        out = np.zeros(r.shape)
        out[pos] = -p[0] * mtn_cor_dx(1.5, r[pos] / p[1]) * r[pos] / (p[1] * p[1])
        return out
    raise ValueError("unknown kernel id")


@dataclass
class KernelMatrix:
    """``KernelMatrix`` (src/structstypes.jl:2-23): lazy A[i,j] = k(x1[i], x2[j], parms)."""
    x1: np.ndarray
    x2: np.ndarray
    parms: np.ndarray
    kid: int
    deriv: Optional[int] = None  # None: the kernel itself; j: its derivative in parameter j

    @property
    def shape(self):
        return (len(self.x1), len(self.x2))

    def block(self, rows, cols) -> np.ndarray:
        """``getindex`` (src/baseoverloads.jl:10-16)."""
        a, b = self.x1[rows], self.x2[cols]
        if a.ndim == 1:
            a = a[None, :]
        if b.ndim == 1:
            b = b[None, :]
        if self.deriv is None:
            return kernel_block(self.kid, a, b, self.parms)
        return dkernel_block(self.kid, self.deriv, a, b, self.parms)

    def row(self, i: int) -> np.ndarray:
        return self.block(slice(i, i + 1), slice(None))[0]

    def col(self, j: int) -> np.ndarray:
        return self.block(slice(None), slice(j, j + 1))[:, 0]

    def full(self) -> np.ndarray:
        """``full`` (src/baseoverloads.jl:20-29)."""
        return self.block(slice(None), slice(None))

    def submatrix(self, ix) -> "KernelMatrix":
        """``submatrix(K, v)`` (src/utils.jl:27-33), ix = 1-based inclusive (a, b, c, d)."""
        a, b, c, d = ix
        return KernelMatrix(self.x1[a - 1:b], self.x2[c - 1:d], self.parms, self.kid, self.deriv)


# ----------------------------------------------------------------------------------------------
# ACA and Nystrom: src/factorizations.jl, src/utils.jl
# ----------------------------------------------------------------------------------------------


def restrictedmaxabs(x: np.ndarray, noinds: set) -> Tuple[float, int]:
    """``restrictedmaxabs`` (src/utils.jl:2-15), 0-based index, strict '>' keeps the first max."""
    n = len(x)
    ind = 0
    while ind in noinds and ind < n - 1:
        ind += 1
    val = 0.0
    ax = np.abs(x)
    for j in range(ind, n):
        if ax[j] > abs(val) and j not in noinds:
            ind = j
            val = float(x[j])
    return val, ind


def ACA(M: KernelMatrix, rtol: float, maxrank: int = 0) -> Tuple[np.ndarray, np.ndarray, List[int], List[int]]:
    """``ACA`` (src/factorizations.jl:9-84).  Returns U, V and the row/column pivot sequences.

    The residual updates are a multiply then a subtract (no fused multiply-add), as in Julia's
    ``tmprow .-= U[j][mi]*V[j]``."""
    nro, ncl = M.shape
    maxsz = min(nro, ncl) if maxrank == 0 else min(maxrank, min(nro, ncl))
    U: List[np.ndarray] = []
    V: List[np.ndarray] = []
    strt = 0
    tmprow = M.row(strt)
    while np.max(np.abs(tmprow)) == 0.0 and strt + 1 < maxsz:
        strt += 1
        tmprow = M.row(strt)
    if strt + 1 == maxsz:
        raise RuntimeError("Incompatible maxrank or matrix dimensions.")
    ucol: set = set()
    urow = {strt}
    rows, cols = [strt], []
    mv, mi = restrictedmaxabs(tmprow, ucol)
    tmprow = tmprow / mv
    tmpcol = M.col(mi)
    U.append(tmpcol)
    V.append(tmprow)
    cols.append(mi)
    znorm2 = float(np.sum(tmprow * tmprow)) * float(np.sum(tmpcol * tmpcol))
    ucol.add(mi)
    frnk = 1
    while np.linalg.norm(tmprow) * np.linalg.norm(tmpcol) > rtol * math.sqrt(znorm2) and frnk < maxsz:
        mv, mi = restrictedmaxabs(tmpcol, urow)
        urow.add(mi)
        rows.append(mi)
        tmprow = M.row(mi)
        for j in range(frnk):
            tmprow = tmprow - U[j][mi] * V[j]
        mv, mi = restrictedmaxabs(tmprow, ucol)
        if mv == 0.0:
            rows.pop()
            break
        ucol.add(mi)
        cols.append(mi)
        tmprow = tmprow / mv
        tmpcol = M.col(mi)
        for j in range(frnk):
            tmpcol = tmpcol - V[j][mi] * U[j]
        for j in range(frnk):
            znorm2 += 2.0 * abs(float(np.dot(U[j], tmpcol))) * abs(float(np.dot(V[j], tmprow)))
        znorm2 += float(np.sum(tmprow * tmprow)) * float(np.sum(tmpcol * tmpcol))
        frnk += 1
        V.append(tmprow)
        U.append(tmpcol)
    return np.stack(U, axis=1), np.stack(V, axis=1), rows, cols


def nystrom_landmarks(n: int, r: int) -> np.ndarray:
    """``Int64.(round.(LinRange(1, n, r)))`` (src/HODLR/src/constructor.jl:31), 0-based.

    LinRange element i is (1-t)*1 + t*n with t = (i-1)/(r-1); Julia rounds ties to even."""
    t = np.arange(r, dtype=np.float64) / float(r - 1)
    vals = (1.0 - t) * 1.0 + t * float(n)
    return np.rint(vals).astype(np.int64) - 1


# ----------------------------------------------------------------------------------------------
# HODLR containers and constructor: src/HODLR/src/structstypes.jl:40-92, constructor.jl:6-95
# ----------------------------------------------------------------------------------------------


@dataclass
class LowRankW:
    """``LowRankW`` = I + M X M' (src/HODLR/src/structstypes.jl:40-43)."""
    M: np.ndarray
    X: np.ndarray  # lower triangular

    def solterm(self, v):
        """``lrx_solterm`` (src/HODLR/src/utils.jl:37-41)."""
        luf = self.X + np.eye(self.X.shape[0])
        Xv = self.X @ v
        return Xv - self.X @ sla.solve_triangular(luf, Xv, lower=True, check_finite=False)

    def solterm_t(self, v):
        """``lrx_solterm_t`` (src/HODLR/src/utils.jl:43-47)."""
        luf = self.X.T + np.eye(self.X.shape[0])
        Xv = self.X.T @ v
        return Xv - self.X.T @ sla.solve_triangular(luf, Xv, lower=False, check_finite=False)

    def ldiv_inplace(self, t):
        """``ldiv!(W, target)`` (src/HODLR/src/baseoverloads.jl:60-63)."""
        t -= self.M @ self.solterm(self.M.T @ t)
        return t

    def ldiv_t_inplace(self, t):
        """``ldiv!(W', target)`` (baseoverloads.jl:65-69)."""
        t -= self.M @ self.solterm_t(self.M.T @ t)
        return t

    def mul(self, src):
        """``mul!(target, W, src)`` (baseoverloads.jl:36-45)."""
        return self.M @ (self.X @ (self.M.T @ src)) + src

    def mul_t(self, src):
        """``mul!(target, W', src)`` (baseoverloads.jl:47-58)."""
        return self.M @ (self.X.T @ (self.M.T @ src)) + src

    def det(self) -> float:
        """``det(W)`` = det(I + M'M X) (baseoverloads.jl:26-28)."""
        return float(np.linalg.det(np.eye(self.X.shape[0]) + (self.M.T @ self.M) @ self.X))

    def full(self):
        """``full(W)`` (baseoverloads.jl:309-311)."""
        return np.eye(self.M.shape[0]) + (self.M @ self.X) @ self.M.T


def lrsymfact(U12: np.ndarray, U21: np.ndarray) -> LowRankW:
    """``lrsymfact`` (src/HODLR/src/utils.jl:29-35): Householder QR of both panels, then
    X = cholesky([I R1R2'; R2R1' I]).L - I and M = blockdiag(Q1, Q2)."""
    Q1, R1 = np.linalg.qr(U12, mode="reduced")
    Q2, R2 = np.linalg.qr(U21, mode="reduced")
    C = R1 @ R2.T
    k1, k2 = C.shape
    big = np.block([[np.eye(k1), C], [C.T, np.eye(k2)]])
    X = np.linalg.cholesky(big) - np.eye(k1 + k2)
    M = np.zeros((Q1.shape[0] + Q2.shape[0], Q1.shape[1] + Q2.shape[1]))
    M[:Q1.shape[0], :Q1.shape[1]] = Q1
    M[Q1.shape[0]:, Q1.shape[1]:] = Q2
    return LowRankW(M, X)


@dataclass
class FactorHODLR:
    """``FactorHODLR`` (src/HODLR/src/structstypes.jl:46-49)."""
    leafW: List[np.ndarray]
    nonleafW: List[List[LowRankW]]


@dataclass
class KernelHODLR:
    """``KernelHODLR`` (src/HODLR/src/structstypes.jl:52-63)."""
    ep: float
    lvl: int
    mrnk: int
    leafindices: list
    nonleafindices: list
    U: Optional[list]
    V: Optional[list]
    L: List[np.ndarray]
    W: Optional[FactorHODLR]
    nys: bool
    pivots: Optional[list] = None  # ACA (rows, cols) per block, kept for parity tests

    @property
    def n(self) -> int:
        return sum(x.shape[0] for x in self.L)


def mapf(f, v, pool=None) -> list:
    """``mapf(f, v, plel)`` (src/HODLR/src/utils.jl:5-8): a map over independent items, run on the
    thread pool ``pool`` when given (the reference's ``plel = true`` with ``ThreadedEx``), else in
    order.  NumPy releases the interpreter lock inside its LAPACK/BLAS calls, so with one BLAS
    thread per worker (the reference's ``BLAS.set_num_threads(1)``, test/runtests.jl:9) the items
    run concurrently.  The result of every item is the same either way."""
    items = list(v)
    if pool is None:
        return [f(x) for x in items]
    return list(pool.map(f, items))


def foreachf(f, v, pool=None) -> None:
    """``foreachf(f, v, plel)`` (src/HODLR/src/utils.jl:10-13)."""
    mapf(f, v, pool)


def build_hodlr(K: KernelMatrix, ep: float, maxrank: int, lvl, nystrom: bool = False, pool=None) -> KernelHODLR:
    """``KernelHODLR(K, ep, maxrank, lvl; nystrom)`` (src/HODLR/src/constructor.jl:6-58)."""
    n = K.shape[0]
    level, leafinds, nonleafinds = HODLRindices(n, lvl)
    if nystrom:
        if maxrank < 2:
            raise ValueError("Please supply a fixed off-diagonal rank that is >=2.")
        if maxrank >= min(min(x[1] - x[0], x[3] - x[2]) for x in leafinds):
            raise ValueError("Your nystrom rank is too big. Reduce the HODLR level or nystrom rank.")
        nyind = nystrom_landmarks(n, maxrank)
        lnd = K.x1[nyind]
        Spp = kernel_block(K.kid, lnd, lnd, K.parms)
        F = sla.cho_factor(Spp, lower=False, check_finite=False)
    # leaves and blocks: mapf over each list (constructor.jl:39, 47-49)
    leaves = mapf(lambda x: K.submatrix(x).full(), leafinds, pool)

    def one_block(x):
        sub = K.submatrix(x)
        if nystrom:
            # nystrom_uvt (src/factorizations.jl:86-94)
            u = kernel_block(K.kid, sub.x1, lnd, K.parms)
            v = sla.cho_solve(F, kernel_block(K.kid, lnd, sub.x2, K.parms), check_finite=False).T
            pv = None
        else:
            u, v, rr, cc = ACA(sub, ep, maxrank)
            pv = (rr, cc)
        return np.ascontiguousarray(u), np.ascontiguousarray(v), pv

    U, V, piv = [], [], []
    for j in range(level):
        res = mapf(one_block, nonleafinds[j], pool)
        U.append([x[0] for x in res])
        V.append([x[1] for x in res])
        piv.append([x[2] for x in res])
    return KernelHODLR(ep, level, maxrank, leafinds, nonleafinds, U, V, leaves, None, nystrom, piv)


def _bdiag_ldiv_lower(Ls: Sequence[np.ndarray], target: np.ndarray) -> None:
    """``ldiv!(BDiagonal(LowerTriangular...), target)`` (src/HODLR/src/BlockDiagonal.jl:62-66)."""
    o = 0
    for Lj in Ls:
        m = Lj.shape[0]
        target[o:o + m] = sla.solve_triangular(Lj, target[o:o + m], lower=True, check_finite=False)
        o += m


def invapply(Wvec, Uvec, Vvec) -> None:
    """``invapply!`` (src/HODLR/src/utils.jl:54-65), leaf (lower triangular) or LowRankW blocks."""
    stepsz = len(Wvec) // (2 * len(Uvec))
    i0 = 0
    for Vj, Uj in zip(Vvec, Uvec):
        for blocks, tgt in ((Wvec[i0:i0 + stepsz], Vj), (Wvec[i0 + stepsz:i0 + 2 * stepsz], Uj)):
            if isinstance(blocks[0], LowRankW):
                o = 0
                for W in blocks:
                    m = W.M.shape[0]
                    W.ldiv_inplace(tgt[o:o + m])
                    o += m
            else:
                _bdiag_ldiv_lower(blocks, tgt)
        i0 += 2 * stepsz


def symmetricfactorize(K: KernelHODLR, pool=None) -> None:
    """``symmetricfactorize!`` (src/HODLR/src/symfact.jl:6-49); ``pool`` runs the reference's
    ``plel = true`` maps (leaf factors, invapply! per level, lrsymfact per block) concurrently."""
    LW = mapf(np.linalg.cholesky, K.L, pool)
    foreachf(lambda lv: invapply(LW, K.U[lv], K.V[lv]), range(len(K.U)), pool)
    nonleafW: List[List[LowRankW]] = []
    for lv in range(len(K.U)):
        nonleafW.append(mapf(lambda vu: lrsymfact(vu[0], vu[1]), list(zip(K.V[lv], K.U[lv])), pool))
        foreachf(lambda lev: invapply(nonleafW[lv], K.U[lev], K.V[lev]), range(lv + 1, len(K.U)), pool)
    K.W = FactorHODLR(LW, nonleafW)
    K.U = None
    K.V = None


# ----------------------------------------------------------------------------------------------
# Products, solves, logdet: src/HODLR/src/baseoverloads.jl:95-209
# ----------------------------------------------------------------------------------------------


def _bdiag_apply(blocks, src, fn):
    out = np.empty_like(src)
    o = 0
    for B in blocks:
        m = B.shape[0] if isinstance(B, np.ndarray) else B.M.shape[0]
        out[o:o + m] = fn(B, src[o:o + m])
        o += m
    return out


def factor_mul(W: FactorHODLR, src: np.ndarray) -> np.ndarray:
    """``mul!(target, W::FactorHODLR, src)`` (baseoverloads.jl:95-109)."""
    tmp = src.copy()
    for j in range(len(W.nonleafW) - 1, -1, -1):
        tmp = _bdiag_apply(W.nonleafW[j], tmp, lambda B, s: B.mul(s))
    return _bdiag_apply(W.leafW, tmp, lambda B, s: B @ s)


def factor_mul_t(W: FactorHODLR, src: np.ndarray) -> np.ndarray:
    """``mul!(target, W'::FactorHODLR, src)`` (baseoverloads.jl:111-124)."""
    tmp = _bdiag_apply(W.leafW, src, lambda B, s: B.T @ s)
    for j in range(len(W.nonleafW)):
        tmp = _bdiag_apply(W.nonleafW[j], tmp, lambda B, s: B.mul_t(s))
    return tmp


def factor_ldiv(W: FactorHODLR, src: np.ndarray) -> np.ndarray:
    """``ldiv!(target, W::FactorHODLR, src)`` (baseoverloads.jl:126-137)."""
    t = np.array(src, dtype=np.float64, copy=True)
    _bdiag_ldiv_lower(W.leafW, t)
    for lvW in W.nonleafW:
        o = 0
        for B in lvW:
            m = B.M.shape[0]
            B.ldiv_inplace(t[o:o + m])
            o += m
    return t


def factor_ldiv_t(W: FactorHODLR, src: np.ndarray) -> np.ndarray:
    """``ldiv!(target, W'::FactorHODLR, src)`` (baseoverloads.jl:139-150)."""
    t = np.array(src, dtype=np.float64, copy=True)
    for lvW in reversed(W.nonleafW):
        o = 0
        for B in lvW:
            m = B.M.shape[0]
            B.ldiv_t_inplace(t[o:o + m])
            o += m
    o = 0
    for Lj in W.leafW:
        m = Lj.shape[0]
        t[o:o + m] = sla.solve_triangular(Lj, t[o:o + m], lower=True, trans="T", check_finite=False)
        o += m
    return t


def hodlr_mul(K: KernelHODLR, src: np.ndarray) -> np.ndarray:
    """``mul!(target, K::KernelHODLR, src)`` (baseoverloads.jl:152-179); src may have columns."""
    if K.W is None:
        tgt = np.zeros_like(src, dtype=np.float64)
        for j, Lj in enumerate(K.L):
            c, d = K.leafindices[j][2:4]
            tgt[c - 1:d] = Lj @ src[c - 1:d]
        for j in range(len(K.U)):
            for k in range(len(K.U[j])):
                a, b, c, d = K.nonleafindices[j][k]
                tgt[c - 1:d] += K.V[j][k] @ (K.U[j][k].T @ src[a - 1:b])
                tgt[a - 1:b] += K.U[j][k] @ (K.V[j][k].T @ src[c - 1:d])
        return tgt
    return factor_mul(K.W, factor_mul_t(K.W, src))


def hodlr_ldiv(K: KernelHODLR, src: np.ndarray) -> np.ndarray:
    """``ldiv!(target, K::KernelHODLR, src)`` (baseoverloads.jl:181-192); ``\\`` (:252-263)."""
    if K.W is None:
        raise RuntimeError("No solves without factorization.")
    return factor_ldiv_t(K.W, factor_ldiv(K.W, src))


def hodlr_logdet(K: KernelHODLR) -> float:
    """``logdet(K::KernelHODLR)`` (baseoverloads.jl:194-209)."""
    if K.W is None:
        raise RuntimeError("No logdet without factorization.")
    out = 0.0
    for Lj in K.L:
        out += 2.0 * float(np.sum(np.log(np.diag(np.linalg.cholesky(Lj)))))
    for lvW in K.W.nonleafW:
        for B in lvW:
            out += 2.0 * math.log(abs(B.det()))
    return out


def hodlr_full(K: KernelHODLR) -> np.ndarray:
    """``full(K::KernelHODLR)`` before factorisation (baseoverloads.jl:313-326)."""
    n = K.n
    out = np.empty((n, n))
    for j, pt in enumerate(K.leafindices):
        out[pt[0] - 1:pt[1], pt[2] - 1:pt[3]] = K.L[j]
    for lev in range(len(K.U)):
        for j in range(len(K.U[lev])):
            a, b, c, d = K.nonleafindices[lev][j]
            out[a - 1:b, c - 1:d] = K.U[lev][j] @ K.V[lev][j].T
            out[c - 1:d, a - 1:b] = K.V[lev][j] @ K.U[lev][j].T
    return out


def factor_full(W: FactorHODLR) -> np.ndarray:
    """``full(W::FactorHODLR)`` (baseoverloads.jl:329-336)."""
    out = sla.block_diag(*W.leafW)
    for lvW in W.nonleafW:
        out = out @ sla.block_diag(*[B.full() for B in lvW])
    return out


# ----------------------------------------------------------------------------------------------
# Derivative HODLR and stochastic gradient: constructor.jl:66-95, utils.jl:67-90,
# baseoverloads.jl:216-234, stochasticgradient.jl:2-44, maxlikfunctions.jl:2-50
# ----------------------------------------------------------------------------------------------


@dataclass
class DerivativeBlock:
    """``DerivativeBlock`` (src/HODLR/src/structstypes.jl:67-72)."""
    K1p: np.ndarray
    K1pd: np.ndarray
    Kp2: np.ndarray
    Kp2d: np.ndarray


@dataclass
class DerivativeHODLR:
    """``DerivativeHODLR`` (structstypes.jl:83-92)."""
    leafindices: list
    nonleafindices: list
    L: List[np.ndarray]
    B: List[List[DerivativeBlock]]
    S: tuple   # cho_factor of K(P, P)
    Sj: np.ndarray


def derivative_hodlr(K: KernelMatrix, j: int, HK: KernelHODLR) -> DerivativeHODLR:
    """``DerivativeHODLR(K, dfun, HK)`` (constructor.jl:66-95); dfun = derivative in parameter j."""
    if not HK.nys:
        raise RuntimeError("This is only valid for Nystrom-block matrices.")
    lnd = K.x1[nystrom_landmarks(K.shape[0], HK.mrnk)]
    S = sla.cho_factor(kernel_block(K.kid, lnd, lnd, K.parms), lower=False, check_finite=False)
    Sj = dkernel_block(K.kid, j, lnd, lnd, K.parms)
    dK = KernelMatrix(K.x1, K.x2, K.parms, K.kid, deriv=j)
    leaves = [dK.submatrix(x).full() for x in HK.leafindices]
    B = []
    for lev in range(HK.lvl):
        Bl = []
        for x in HK.nonleafindices[lev]:
            a, b, c, d = x
            x1, x2 = K.x1[a - 1:b], K.x2[c - 1:d]
            # DBlock (src/HODLR/src/utils.jl:67-74)
            Bl.append(DerivativeBlock(kernel_block(K.kid, x1, lnd, K.parms),
                                      dkernel_block(K.kid, j, x1, lnd, K.parms),
                                      kernel_block(K.kid, lnd, x2, K.parms),
                                      dkernel_block(K.kid, j, lnd, x2, K.parms)))
        B.append(Bl)
    return DerivativeHODLR(HK.leafindices, HK.nonleafindices, leaves, B, S, Sj)


def _cs(S, v):
    return sla.cho_solve(S, v, check_finite=False)


def dblock_mul(B: DerivativeBlock, src, S, Sj):
    """``DBlock_mul`` (src/HODLR/src/utils.jl:76-82)."""
    out = B.K1pd @ _cs(S, B.Kp2 @ src)
    out = out - B.K1p @ _cs(S, Sj @ _cs(S, B.Kp2 @ src))
    out = out + B.K1p @ _cs(S, B.Kp2d @ src)
    return out


def dblock_mul_t(B: DerivativeBlock, src, S, Sj):
    """``DBlock_mul_t`` (src/HODLR/src/utils.jl:84-90)."""
    out = B.Kp2.T @ _cs(S, B.K1pd.T @ src)
    out = out - B.Kp2.T @ _cs(S, Sj @ _cs(S, B.K1p.T @ src))
    out = out + B.Kp2d.T @ _cs(S, B.K1p.T @ src)
    return out


def derivative_mul(DK: DerivativeHODLR, src: np.ndarray) -> np.ndarray:
    """``mul!(target, DK::DerivativeHODLR, src)`` (baseoverloads.jl:216-234)."""
    tgt = np.zeros_like(src, dtype=np.float64)
    for j, Lj in enumerate(DK.L):
        c, d = DK.leafindices[j][2:4]
        tgt[c - 1:d] += Lj @ src[c - 1:d]
    for lev in range(len(DK.B)):
        for k, B in enumerate(DK.B[lev]):
            a, b, c, d = DK.nonleafindices[lev][k]
            tgt[c - 1:d] += dblock_mul_t(B, src[a - 1:b], DK.S, DK.Sj)
            tgt[a - 1:b] += dblock_mul(B, src[c - 1:d], DK.S, DK.Sj)
    return tgt


def derivative_full(DK: DerivativeHODLR) -> np.ndarray:
    """``full(DK::DerivativeHODLR)`` (baseoverloads.jl:338-351) with ``DBlock_full`` (utils.jl:92-98)."""
    n = sum(x.shape[0] for x in DK.L)
    out = np.zeros((n, n))
    for j, pt in enumerate(DK.leafindices):
        out[pt[0] - 1:pt[1], pt[2] - 1:pt[3]] = DK.L[j]
    for lev in range(len(DK.B)):
        for k, B in enumerate(DK.B[lev]):
            a, b, c, d = DK.nonleafindices[lev][k]
            blk = B.K1pd @ _cs(DK.S, B.Kp2) - B.K1p @ _cs(DK.S, DK.Sj @ _cs(DK.S, B.Kp2)) \
                + B.K1p @ _cs(DK.S, B.Kp2d)
            out[a - 1:b, c - 1:d] = blk
            out[c - 1:d, a - 1:b] = blk.T
    return out


def hodlr_trace_apply(HK: KernelHODLR, DK: DerivativeHODLR, v: np.ndarray) -> float:
    """``HODLR_trace_apply`` (src/HODLR/src/stochasticgradient.jl:2-10)."""
    t1 = factor_ldiv_t(HK.W, v)
    t2 = derivative_mul(DK, t1)
    return float(np.dot(t1, t2))


def hodlr_grad_term(K: KernelMatrix, HK: KernelHODLR, j: int, dat: np.ndarray, vecs) -> float:
    """``HODLR_grad_term`` (stochasticgradient.jl:14-26)."""
    DK = derivative_hodlr(K, j, HK)
    prvec = hodlr_ldiv(HK, derivative_mul(DK, hodlr_ldiv(HK, dat)))
    trtm = sum(hodlr_trace_apply(HK, DK, v) for v in vecs) / len(vecs)
    return 0.5 * (trtm - float(np.dot(dat, prvec)))


def stoch_gradient(K: KernelMatrix, HK: KernelHODLR, dat: np.ndarray, nparams: int, vecs) -> np.ndarray:
    """``stoch_gradient`` (stochasticgradient.jl:30-44) with shuffle=false."""
    if HK.U is not None:
        raise RuntimeError("The matrix needs to be factorized for this to work.")
    return np.array([hodlr_grad_term(K, HK, j, dat, vecs) for j in range(nparams)])


def negloglik(HK: KernelHODLR, dat: np.ndarray) -> float:
    """``negloglik`` (src/HODLR/src/maxlikfunctions.jl:2-9)."""
    if HK.U is not None:
        raise RuntimeError("The HODLR matrix needs to be factorized for this.")
    return 0.5 * hodlr_logdet(HK) + 0.5 * float(np.dot(dat, hodlr_ldiv(HK, dat)))


def nll_objective(prms, grad: Optional[np.ndarray], pts: np.ndarray, dat: np.ndarray, kid: int,
                  rank: int, lvl, saav) -> float:
    """``nll_objective`` (maxlikfunctions.jl:29-50): Nystrom assembly with ep = 0, factorise,
    NLL, and (when ``grad`` has entries) the stochastic gradient."""
    K = KernelMatrix(pts, pts, np.asarray(prms, dtype=np.float64), kid)
    HK = build_hodlr(K, 0.0, rank, lvl, nystrom=True)
    symmetricfactorize(HK)
    nll = negloglik(HK, dat)
    if grad is not None and len(grad) > 0:
        grad[:] = stoch_gradient(K, HK, dat, len(grad), saav)
    return nll


def profile_negloglik(HK: KernelHODLR, dat: np.ndarray) -> float:
    """``profile_negloglik`` (src/HODLR/src/maxlikfunctions.jl:11-19): the NLL with the scale
    parameter profiled out, 0.5*(logdet K + n*log(y' K^-1 y))."""
    if HK.U is not None:
        raise RuntimeError("The HODLR matrix needs to be factorized for this.")
    return 0.5 * (hodlr_logdet(HK) + len(dat) * np.log(float(np.dot(dat, hodlr_ldiv(HK, dat)))))


def scaleparm_mle(HK: KernelHODLR, dat: np.ndarray) -> float:
    """``scaleparm_mle`` / ``nlpl_scale`` (maxlikfunctions.jl:21-27,52-58) on a factorised
    matrix: the profiled scale estimate y' K^-1 y / n."""
    return float(np.dot(dat, hodlr_ldiv(HK, dat))) / len(dat)


def hodlr_p_grad_term(K: KernelMatrix, HK: KernelHODLR, j: int, dat: np.ndarray, vecs) -> float:
    """``HODLR_p_grad_term`` (stochasticgradient.jl:48-64)."""
    DK = derivative_hodlr(K, j, HK)
    prvec = hodlr_ldiv(HK, derivative_mul(DK, hodlr_ldiv(HK, dat)))
    trtm = sum(hodlr_trace_apply(HK, DK, v) for v in vecs) / len(vecs)
    return 0.5 * (trtm - len(dat) * float(np.dot(dat, prvec)) / float(np.dot(dat, hodlr_ldiv(HK, dat))))


def stoch_profile_gradient(K: KernelMatrix, HK: KernelHODLR, dat: np.ndarray, nparams: int, vecs) -> np.ndarray:
    """``stoch_profile_gradient`` (stochasticgradient.jl:68-86) with shuffle=false."""
    if HK.U is not None:
        raise RuntimeError("The matrix needs to be factorized for this to work.")
    return np.array([hodlr_p_grad_term(K, HK, j, dat, vecs) for j in range(nparams)])


def nlpl_objective(prms, grad: Optional[np.ndarray], pts: np.ndarray, dat: np.ndarray, kid: int,
                   rank: int, lvl, saav) -> float:
    """``nlpl_objective`` (maxlikfunctions.jl:61-82): ``nll_objective`` for the profile
    likelihood."""
    K = KernelMatrix(pts, pts, np.asarray(prms, dtype=np.float64), kid)
    HK = build_hodlr(K, 0.0, rank, lvl, nystrom=True)
    symmetricfactorize(HK)
    nll = profile_negloglik(HK, dat)
    if grad is not None and len(grad) > 0:
        grad[:] = stoch_profile_gradient(K, HK, dat, len(grad), saav)
    return nll


def hess_tr1_sym_diag(HK: KernelHODLR, DKj: DerivativeHODLR, v: np.ndarray) -> float:
    """``HODLR_hess_tr1_sym_diag`` (src/HODLR/src/stochastichessian.jl:58-66):
    |W^-1 dK_j W'^-1 v|^2."""
    tp2 = factor_ldiv(HK.W, derivative_mul(DKj, factor_ldiv_t(HK.W, v)))
    return float(np.dot(tp2, tp2))


def hess_tr1_sym_offdiag(HK: KernelHODLR, DKj: DerivativeHODLR, DKk: DerivativeHODLR, v: np.ndarray) -> float:
    """``HODLR_hess_tr1_sym_offdiag`` (stochastichessian.jl:68-77): |W^-1 (dK_j + dK_k) W'^-1 v|^2."""
    tp1 = factor_ldiv_t(HK.W, v)
    tp2 = factor_ldiv(HK.W, derivative_mul(DKj, tp1) + derivative_mul(DKk, tp1))
    return float(np.dot(tp2, tp2))


def stoch_fisher(K: KernelMatrix, HK: KernelHODLR, DKs, vecs) -> np.ndarray:
    """``stoch_fisher`` (stochastichessian.jl:91-115) with shuffle=false: diagonal first, then
    the off-diagonal entries by polarisation."""
    if HK.U is not None:
        raise RuntimeError("The matrix needs to be factorized.")
    m = len(DKs)
    out = np.zeros((m, m))
    for j in range(m):
        out[j, j] = 0.5 * sum(hess_tr1_sym_diag(HK, DKs[j], v) for v in vecs) / len(vecs)
    for j in range(m):
        for k in range(j + 1, m):
            tmp1 = 0.5 * sum(hess_tr1_sym_offdiag(HK, DKs[j], DKs[k], v) for v in vecs) / len(vecs)
            out[j, k] = 0.5 * (tmp1 - out[j, j] - out[k, k])
            out[k, j] = out[j, k]
    return out


def grad_and_fisher_matrix(prms, pts: np.ndarray, dat: np.ndarray, kid: int, rank: int, lvl, saav):
    """``grad_and_fisher_matrix(prm, data, opts)`` (stochastichessian.jl:152-181): the
    stochastic gradient and Fisher matrix of a freshly assembled Nystrom HODLR."""
    K = KernelMatrix(pts, pts, np.asarray(prms, dtype=np.float64), kid)
    HK = build_hodlr(K, 0.0, rank, lvl, nystrom=True)
    symmetricfactorize(HK)
    m = len(prms)
    g = np.zeros(m)
    F = np.zeros((m, m))
    for j in range(m):
        HKj = derivative_hodlr(K, j, HK)
        trace_j = float(np.mean([hodlr_trace_apply(HK, HKj, v) for v in saav]))
        g[j] = 0.5 * (trace_j - float(np.dot(dat, hodlr_ldiv(HK, derivative_mul(HKj, hodlr_ldiv(HK, dat))))))
        for k in range(j, m):
            HKk = derivative_hodlr(K, k, HK)
            if k == j:
                F[j, j] = 0.5 * float(np.mean([hess_tr1_sym_diag(HK, HKj, v) for v in saav]))
            else:
                F[j, k] = 0.25 * float(np.mean([hess_tr1_sym_offdiag(HK, HKj, HKk, v) for v in saav]))
    for j in range(m):
        for k in range(j + 1, m):
            F[j, k] -= 0.5 * (F[j, j] + F[k, k])
            F[k, j] = F[j, k]
    return g, F


# ----------------------------------------------------------------------------------------------
# Stochastic Hessian: constructor.jl:100-121 (second-derivative leaves and blocks),
# utils.jl:100-177 (SBlock, SDBlock_mul, SDBlock_mul_t, Deriv2mul), stochastichessian.jl:3-56,
# 79-89, 117-147 (the solve and trace terms, stoch_hessian)
# ----------------------------------------------------------------------------------------------


def d2kernel_block(kid: int, j: int, k: int, x1: np.ndarray, x2: np.ndarray, p: Sequence[float]) -> np.ndarray:
    """Second derivative of ``kernel_block`` in parameters j and k (0: scale, 1: range, 2: nugget).

    The reference takes these as user functions (``d2funs`` of stoch_hessian,
    stochastichessian.jl:117-121); this is the closed form of the same kernels:
    Matern-3/2, k = p0 (1 + z) e^-z with z = sqrt(3) r / p1: d00 = 0, d01 = z^2 e^-z / p1,
    d11 = p0 z^2 (z - 3) e^-z / p1^2 (0 where r / p1 <= 1e-8, as for the first derivative);
    RQ, k = p0^2 / u^2 with u = 1 + t^2, t = r / p1: d00 = 2 / u^2, d01 = 8 p0 r^2 / (p1^3 u^3),
    d11 = 12 p0^2 r^2 (t^2 - 1) / (p1^4 u^4).  Every pair with the nugget is 0."""
    j, k = min(j, k), max(j, k)
    r, _ = _pairwise(x1, x2)
    if k == 2:
        return np.zeros(r.shape)
    if kid == KERNEL_RQ:
        t = r / p[1]
        u = 1.0 + t * t
        if (j, k) == (0, 0):
            return 2.0 / (u * u)
        if (j, k) == (0, 1):
            return 8.0 * p[0] * r * r / (p[1] ** 3) / (u * u * u)
        return 12.0 * p[0] * p[0] * r * r * (t * t - 1.0) / (p[1] ** 4) / (u ** 4)
    if kid == KERNEL_MATERN32:
        out = np.zeros(r.shape)
        if (j, k) == (0, 0):
            return out
        x = r / p[1]
        m = np.abs(x) > 1.0e-8
        z = SQRT3 * x[m]
        e = np.exp(-z)
        if (j, k) == (0, 1):
            out[m] = z * z * e / p[1]
        else:
            out[m] = p[0] * z * z * (z - 3.0) * e / (p[1] * p[1])
        return out
    raise ValueError("unknown kernel id")


def d2_is_zero(kid: int, j: int, k: int) -> bool:
    """Pairs whose second derivative vanishes identically (``ZeroFunction`` in stoch_hessian)."""
    j, k = min(j, k), max(j, k)
    return k == 2 or (kid == KERNEL_MATERN32 and (j, k) == (0, 0))


@dataclass
class SecondDerivativeBlock:
    """``SecondDerivativeBlock`` (src/HODLR/src/structstypes.jl:77-80)."""
    K1pjk: np.ndarray
    Kp2jk: np.ndarray


def second_derivative_parts(K: KernelMatrix, HK: KernelHODLR, j: int, k: int):
    """``SecondDerivativeBlocks`` and ``SecondDerivativeLeaves`` (constructor.jl:100-121) and
    ``Sjk`` (HODLR_hess_extra, stochastichessian.jl:33-47): the d2 blocks K(x1, P), K(P, x2) of every non-leaf block,
    the dense d2 leaves, and d2 K(P, P)."""
    lnd = K.x1[nystrom_landmarks(K.shape[0], HK.mrnk)]
    blocks = []
    for lev in range(HK.lvl):
        Bl = []
        for x in HK.nonleafindices[lev]:
            a, b, c, d = x
            Bl.append(SecondDerivativeBlock(d2kernel_block(K.kid, j, k, K.x1[a - 1:b], lnd, K.parms),
                                            d2kernel_block(K.kid, j, k, lnd, K.x2[c - 1:d], K.parms)))
        blocks.append(Bl)
    leaves = []
    for x in HK.leafindices:
        a, b, c, d = x
        leaves.append(d2kernel_block(K.kid, j, k, K.x1[a - 1:b], K.x2[c - 1:d], K.parms))
    Sjk = d2kernel_block(K.kid, j, k, lnd, lnd, K.parms)
    return blocks, leaves, Sjk


def sdblock_mul(Bj: DerivativeBlock, Bk: DerivativeBlock, Bjk: SecondDerivativeBlock, src, S, Spj, Spk, Spjk):
    """``SDBlock_mul`` (src/HODLR/src/utils.jl:110-132), term for term (the reference's own terms,
    which are not the second derivative of a Nystrom block; see the design notes)."""
    out = Bjk.K1pjk @ _cs(S, Bj.Kp2 @ src)
    out = out - Bj.K1pd @ _cs(S, Spk @ _cs(S, Bj.Kp2 @ src))
    out = out + Bj.K1pd @ _cs(S, Bk.Kp2d @ src)
    out = out + Bk.K1pd @ _cs(S, Spj @ _cs(S, Bj.Kp2 @ src))
    out = out - Bk.K1p @ _cs(S, Spk @ _cs(S, Spj @ _cs(S, Bk.Kp2 @ src)))
    out = out + Bk.K1p @ _cs(S, Spjk @ _cs(S, Bk.Kp2 @ src))
    out = out - Bk.K1p @ _cs(S, Spj @ _cs(S, Spk @ _cs(S, Bk.Kp2 @ src)))
    out = out + Bk.K1p @ _cs(S, Spj @ _cs(S, Bj.Kp2d @ src))
    out = out + Bk.K1pd @ _cs(S, Bk.Kp2 @ src)
    out = out - Bk.K1p @ _cs(S, Spk @ _cs(S, Bk.Kp2 @ src))
    out = out + Bk.K1p @ _cs(S, Bjk.Kp2jk @ src)
    return out


def sdblock_mul_t(Bj: DerivativeBlock, Bk: DerivativeBlock, Bjk: SecondDerivativeBlock, src, S, Spj, Spk, Spjk):
    """``SDBlock_mul_t`` (utils.jl:134-155), term for term (t_mul(A, x) = A' x)."""
    out = Bj.Kp2.T @ _cs(S, Bjk.K1pjk.T @ src)
    out = out - Bj.Kp2.T @ _cs(S, Spk @ _cs(S, Bj.K1pd.T @ src))
    out = out + Bk.Kp2d.T @ _cs(S, Bk.K1pd.T @ src)
    out = out + Bj.Kp2.T @ _cs(S, Spj @ _cs(S, Bk.K1pd.T @ src))
    out = out - Bj.Kp2.T @ _cs(S, Spj @ _cs(S, Spk @ _cs(S, Bk.K1p.T @ src)))
    out = out + Bj.Kp2.T @ _cs(S, Spjk @ _cs(S, Bk.K1p.T @ src))
    out = out - Bj.Kp2.T @ _cs(S, Spk @ _cs(S, Spj @ _cs(S, Bk.K1p.T @ src)))
    out = out + Bk.Kp2d.T @ _cs(S, Spj @ _cs(S, Bk.K1p.T @ src))
    out = out + Bj.Kp2d.T @ _cs(S, Bk.K1pd.T @ src)
    out = out - Bj.Kp2d.T @ _cs(S, Spk @ _cs(S, Bk.K1p.T @ src))
    out = out + Bjk.Kp2jk.T @ _cs(S, Bk.K1p.T @ src)
    return out


def deriv2mul(DKj: DerivativeHODLR, DKk: DerivativeHODLR, D2B2, D2BL, Sjk, src: np.ndarray) -> np.ndarray:
    """``Deriv2mul`` (utils.jl:157-177): the d2 leaves, then per non-leaf block SDBlock_mul_t into
    the column range and SDBlock_mul into the row range."""
    tgt = np.zeros_like(src, dtype=np.float64)
    for q, Lq in enumerate(D2BL):
        c, d = DKj.leafindices[q][2:4]
        tgt[c - 1:d] += Lq @ src[c - 1:d]
    for lev in range(len(DKj.B)):
        for q in range(len(DKj.B[lev])):
            a, b, c, d = DKj.nonleafindices[lev][q]
            Bj, Bk, Bjk = DKj.B[lev][q], DKk.B[lev][q], D2B2[lev][q]
            tgt[c - 1:d] += sdblock_mul_t(Bj, Bk, Bjk, src[a - 1:b], DKj.S, DKj.Sj, DKk.Sj, Sjk)
            tgt[a - 1:b] += sdblock_mul(Bj, Bk, Bjk, src[c - 1:d], DKj.S, DKj.Sj, DKk.Sj, Sjk)
    return tgt


def hess_slv(HK: KernelHODLR, DKj, DKk, D2B2, D2BL, Sjk, data, HKsd) -> float:
    """``HODLR_hess_slv`` (stochastichessian.jl:3-13)."""
    out = -hodlr_ldiv(HK, derivative_mul(DKk, hodlr_ldiv(HK, derivative_mul(DKj, HKsd))))
    out = out - hodlr_ldiv(HK, derivative_mul(DKj, hodlr_ldiv(HK, derivative_mul(DKk, HKsd))))
    out = out + hodlr_ldiv(HK, deriv2mul(DKj, DKk, D2B2, D2BL, Sjk, HKsd))
    return float(np.dot(data, out))


def hess_slv_no2d(HK: KernelHODLR, DKj, DKk, data, HKsd) -> float:
    """``HODLR_hess_slv_no2d`` (stochastichessian.jl:50-56)."""
    out = -hodlr_ldiv(HK, derivative_mul(DKk, hodlr_ldiv(HK, derivative_mul(DKj, HKsd))))
    out = out - hodlr_ldiv(HK, derivative_mul(DKj, hodlr_ldiv(HK, derivative_mul(DKk, HKsd))))
    return float(np.dot(data, out))


def p_hess_slv(HK: KernelHODLR, DKj, DKk, parts, data, HKsd, dotm) -> float:
    """``HODLR_p_hess_slv`` (stochastichessian.jl:15-31): the solve term of the profile likelihood,
    n * (data'out / dotm + (data' K^-1 dK_j u)(data' K^-1 dK_k u) / dotm^2) with
    out = -K^-1 dK_k K^-1 dK_j u - K^-1 dK_j K^-1 dK_k u + K^-1 D2_jk u, u = K^-1 data and
    dotm = data'u.  ``parts`` = (D2B2, D2BL, Sjk), or None for a second derivative that is zero
    (the reference's general path with a zero function: the D2 term vanishes)."""
    tmp1 = derivative_mul(DKj, HKsd)
    tmp2 = derivative_mul(DKk, HKsd)
    out = -hodlr_ldiv(HK, derivative_mul(DKk, hodlr_ldiv(HK, tmp1)))
    out = out - hodlr_ldiv(HK, derivative_mul(DKj, hodlr_ldiv(HK, tmp2)))
    if parts is not None:
        out = out + hodlr_ldiv(HK, deriv2mul(DKj, DKk, parts[0], parts[1], parts[2], HKsd))
    ret = float(np.dot(data, out)) / dotm
    t2 = float(np.dot(data, hodlr_ldiv(HK, tmp1))) / (dotm * dotm)
    t2 *= float(np.dot(data, hodlr_ldiv(HK, tmp2)))
    return len(data) * (ret + t2)


def hess_tr2(HK: KernelHODLR, DKj, DKk, D2B2, D2BL, Sjk, v) -> float:
    """``HODLR_hess_tr2`` (stochastichessian.jl:79-89): tp1 = W'^-1 v, tp1 . Deriv2mul(tp1)."""
    tp1 = factor_ldiv_t(HK.W, v)
    return float(np.dot(tp1, deriv2mul(DKj, DKk, D2B2, D2BL, Sjk, tp1)))


def stoch_hessian(K: KernelMatrix, HK: KernelHODLR, dat: np.ndarray, vecs, profile: bool = False) -> np.ndarray:
    """``stoch_hessian`` (stochastichessian.jl:117-147) with shuffle = false: minus the
    stochastic Fisher matrix, plus for every pair j <= k the solve term (with the
    second-derivative product where the second derivative is not identically zero, otherwise
    ``HODLR_hess_slv_no2d``) and the trace term (``HODLR_hess_extra``, :33-47).  With
    ``profile`` (nlpl_hessian, maxlikfunctions.jl:120-136) the solve term is
    ``HODLR_p_hess_slv``; the reference raises for a ``ZeroFunction`` pair there, and such pairs
    take its general path with a zero second derivative instead (no D2 term, zero trace term).
    Returns the symmetric matrix of the upper triangle."""
    if HK.U is not None:
        raise RuntimeError("The matrix needs to be factorized.")
    m = len(K.parms)
    DKs = [derivative_hodlr(K, j, HK) for j in range(m)]
    out = -stoch_fisher(K, HK, DKs, vecs)
    HKsd = hodlr_ldiv(HK, dat)
    dotm = float(np.dot(dat, HKsd))
    for j in range(m):
        for k in range(j, m):
            if profile:
                parts = None if d2_is_zero(K.kid, j, k) else second_derivative_parts(K, HK, j, k)
                sterm = p_hess_slv(HK, DKs[j], DKs[k], parts, dat, HKsd, dotm)
                t2 = 0.0 if parts is None else sum(hess_tr2(HK, DKs[j], DKs[k], *parts, v) for v in vecs) / len(vecs)
                out[j, k] += 0.5 * t2 - 0.5 * sterm
            elif not d2_is_zero(K.kid, j, k):
                D2B2, D2BL, Sjk = second_derivative_parts(K, HK, j, k)
                sterm = hess_slv(HK, DKs[j], DKs[k], D2B2, D2BL, Sjk, dat, HKsd)
                t2 = sum(hess_tr2(HK, DKs[j], DKs[k], D2B2, D2BL, Sjk, v) for v in vecs) / len(vecs)
                out[j, k] += 0.5 * t2 - 0.5 * sterm
            else:
                out[j, k] -= 0.5 * hess_slv_no2d(HK, DKs[j], DKs[k], dat, HKsd)
    return np.triu(out) + np.triu(out, 1).T


def kd_order(pts: np.ndarray, leaf: int = 32) -> np.ndarray:
    """k-d ordering checked against the GPU's ``km_kd_order``.  The reference sorts with
    NearestNeighbors 0.4.9 ``KDTree(pts).data`` (src/HODLR/src/constructor.jl:180), a third-party
    permutation that is not reproduced (parity unpinned against it); this is the build's own
    rule: a range of more than ``leaf`` points is sorted stably on the coordinate of larger spread
    (max - min, x on a tie), split at floor(len/2), and both halves ordered the same way."""
    pts = np.asarray(pts, dtype=np.float64).reshape(-1, 2)
    out = np.arange(len(pts), dtype=np.int64)

    def rec(lo: int, hi: int) -> None:
        if hi - lo <= leaf:
            return
        seg = out[lo:hi]
        sub = pts[seg]
        ax = 0 if (sub[:, 0].max() - sub[:, 0].min()) >= (sub[:, 1].max() - sub[:, 1].min()) else 1
        out[lo:hi] = seg[np.argsort(sub[:, ax], kind="stable")]
        h = (hi - lo) // 2
        rec(lo, lo + h)
        rec(lo + h, hi)

    import sys
    old = sys.getrecursionlimit()
    sys.setrecursionlimit(max(old, 10000))
    try:
        rec(0, len(pts))
    finally:
        sys.setrecursionlimit(old)
    return out


@dataclass
class RKernelHODLR:
    """``RKernelHODLR`` (src/HODLR/src/structstypes.jl:22-27): A11 and A22 dense or recursive,
    A12 and A21 as (U, V, row pivots, column pivots) from ACA."""
    A11: object
    A22: object
    A12: tuple
    A21: tuple


def rkernel_hodlr(K: KernelMatrix, tol: float, maxrank: int = 0, lvl=None):
    """``RKernelHODLR(K, tol, maxrank, lvl)`` (src/HODLR/src/constructor.jl:130-161)."""
    lvl = LogLevel(7) if lvl is None else lvl
    if isinstance(lvl, LogLevel):
        return rkernel_hodlr(K, tol, maxrank, FixedLevel(_floor_log2(min(K.shape)) - lvl.lv))
    if lvl.lv == 0:
        return K.full()
    len1, len2 = K.shape
    m1, m2 = len1 // 2, len2 // 2

    def sub(a, b, c, d):
        return KernelMatrix(K.x1[a:b], K.x2[c:d], K.parms, K.kid, K.deriv)

    K11, K22 = sub(0, m1, 0, m2), sub(m1, len1, m2, len2)
    A12 = ACA(sub(0, m1, m2, len2), tol, maxrank)
    A21 = ACA(sub(m1, len1, 0, m2), tol, maxrank)
    if lvl.lv == 1:
        return RKernelHODLR(K11.full(), K22.full(), A12, A21)
    return RKernelHODLR(rkernel_hodlr(K11, tol, maxrank, FixedLevel(lvl.lv - 1)),
                        rkernel_hodlr(K22, tol, maxrank, FixedLevel(lvl.lv - 1)), A12, A21)


def rhodlr_shape(R) -> Tuple[int, int]:
    """``size(R)`` (src/HODLR/src/baseoverloads.jl:297-299)."""
    if isinstance(R, np.ndarray):
        return R.shape
    a, b = rhodlr_shape(R.A11), rhodlr_shape(R.A22)
    return a[0] + b[0], a[1] + b[1]


def rhodlr_mul(R, v: np.ndarray) -> np.ndarray:
    """``*(R::RKernelHODLR, V)`` (src/HODLR/src/baseoverloads.jl:301-305), UVt products as
    U (V' v) (:295)."""
    if isinstance(R, np.ndarray):
        return R @ v
    c1 = rhodlr_shape(R.A11)[1]
    v1, v2 = v[:c1], v[c1:]
    top = rhodlr_mul(R.A11, v1) + R.A12[0] @ (R.A12[1].T @ v2)
    bot = R.A21[0] @ (R.A21[1].T @ v1) + rhodlr_mul(R.A22, v2)
    return np.concatenate([top, bot])


def rhodlr_blocks(R) -> list:
    """Off-diagonal blocks in recursive order: A12, A21, then those of A11, then of A22."""
    if isinstance(R, np.ndarray):
        return []
    return [R.A12, R.A21] + rhodlr_blocks(R.A11) + rhodlr_blocks(R.A22)


# ----------------------------------------------------------------------------------------------
# Dense oracle: src/HODLR/src/exactmaxlik.jl
# ----------------------------------------------------------------------------------------------


def dense_nll(K: KernelMatrix, dat: np.ndarray) -> float:
    """``exact_nll_objective`` NLL part (exactmaxlik.jl:2-17)."""
    F = sla.cho_factor(K.full(), lower=False, check_finite=False)
    logdet = 2.0 * float(np.sum(np.log(np.diag(F[0]))))
    return 0.5 * logdet + 0.5 * float(np.dot(dat, sla.cho_solve(F, dat, check_finite=False)))


def dense_gradient(K: KernelMatrix, dat: np.ndarray, nparams: int) -> np.ndarray:
    """``exact_gradient_term`` (exactmaxlik.jl:42-48) for each parameter."""
    F = sla.cho_factor(K.full(), lower=False, check_finite=False)
    out = np.zeros(nparams)
    a = sla.cho_solve(F, dat, check_finite=False)
    for j in range(nparams):
        dK = KernelMatrix(K.x1, K.x2, K.parms, K.kid, deriv=j).full()
        out[j] = 0.5 * np.trace(sla.cho_solve(F, dK, check_finite=False)) - 0.5 * float(a @ (dK @ a))
    return out


def hodlr_exact_gradient(K: KernelMatrix, rank: int, lvl, dat: np.ndarray, nparams: int) -> np.ndarray:
    """``exact_HODLR_gradient`` (exactmaxlik.jl:62-80): exact gradient of the Nystrom-HODLR NLL,
    0.5*(tr(HK^-1 dHK) - y' HK^-1 dHK HK^-1 y), with dense matrices (small n only)."""
    HK = build_hodlr(K, 0.0, rank, lvl, nystrom=True)
    HKf = sla.cho_factor(hodlr_full(HK), lower=False, check_finite=False)
    out = np.zeros(nparams)
    a = sla.cho_solve(HKf, dat, check_finite=False)
    for j in range(nparams):
        dK = derivative_full(derivative_hodlr(K, j, HK))
        out[j] = 0.5 * (np.trace(sla.cho_solve(HKf, dK, check_finite=False)) - float(a @ (dK @ a)))
    return out


def _splitmix64_mix(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser (Steele, Lea and Flood, OOPSLA 2014) on uint64 arrays (wrapping)."""
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def rademacher_probes(n: int, p: int, seed: int) -> np.ndarray:
    """The engine's seeded probe block (n x p): entry (i, j) = +1 when the top bit of
    SplitMix64(SplitMix64(seed) + j*n + i) is set, else -1.  It stands in for ``givesaa``
    (src/HODLR/src/utils.jl:22-27), whose Julia generator is not reproduced."""
    base = _splitmix64_mix(np.array([seed], dtype=np.uint64))[0]
    with np.errstate(over="ignore"):
        e = base + np.arange(n * p, dtype=np.uint64)
    bits = _splitmix64_mix(e) >> np.uint64(63)
    return np.where(bits == 1, 1.0, -1.0).reshape(p, n).T.copy()


def givesaa(length: int, sz: int, seed: int) -> List[np.ndarray]:
    """Rademacher probe vectors as ``givesaa`` (src/HODLR/src/utils.jl:22-27) makes them; the
    generator is NumPy's PCG64 from ``seed`` (Julia's Xoshiro stream is not reproduced)."""
    rng = np.random.default_rng(seed)
    return [rng.choice(np.array([-1.0, 1.0]), size=sz) for _ in range(length)]
