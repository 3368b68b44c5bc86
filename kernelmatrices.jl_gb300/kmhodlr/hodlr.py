"""Python mirror of the KernelMatrices.jl HODLR interface, running on the GB300 engine.

Names, argument meanings and errors follow the reference:
  KernelMatrix(pts, pts, parms, kernel)              src/structstypes.jl:17
  FixedLevel(k), LogLevel(k)                         src/HODLR/src/structstypes.jl:30-37
  KernelHODLR(K, ep, maxrank, lvl; nystrom, ...)     src/HODLR/src/constructor.jl:6-58
  symmetricfactorize(HK)   (Julia: symmetricfactorize!)  src/HODLR/src/symfact.jl:6-49
  HK @ x (mul!/*), HK.ldiv(b) / HK \\ b (ldiv!/\\), logdet(HK)   baseoverloads.jl:152-209
  HK.W.ldiv(v), HK.W.T.ldiv(v), HK.W @ v, HK.W.T @ v            baseoverloads.jl:95-150
Errors: PosDefException for non-positive-definite factors, KMError (Julia's ErrorException)
for the rest.  Every operation runs in libkmhodlr.so; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _lib as L


class KMError(RuntimeError):
    """A failed engine call (Julia ``error(...)``)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class PosDefException(KMError):
    """Mirror of Julia's ``LinearAlgebra.PosDefException``."""


def _check(h, rc: int):
    if rc == L.KM_OK:
        return
    lib = L.load()
    msg = lib.km_last_error(h).decode() if h else "error"
    if rc == L.KM_ERR_NOT_SPD:
        raise PosDefException(rc, msg)
    raise KMError(rc, msg)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


@dataclass(frozen=True)
class FixedLevel:
    lv: int


@dataclass(frozen=True)
class LogLevel:
    lv: int


def _level(lvl):
    if isinstance(lvl, FixedLevel):
        return L.KM_LEVEL_FIXED, lvl.lv
    if isinstance(lvl, LogLevel):
        return L.KM_LEVEL_LOG, lvl.lv
    raise TypeError("level must be FixedLevel or LogLevel")


# ---- kernels ----------------------------------------------------------------------------------

@dataclass(frozen=True)
class RatQuad:
    """k(x, y, p) = p1^2 / (1 + (|x-y|/p2)^2)^2 + p3 [x == y]   (README.md:42-48)."""
    kid: int = L.KM_KERNEL_RATQUAD


@dataclass(frozen=True)
class Matern32:
    """k(x, y, p) = p1 (1 + sqrt3 r/p2) exp(-sqrt3 r/p2) + p3 [x == y]
    (mtn_kernfun at nu = 3/2, src/covariancefunctions.jl:258-266)."""
    kid: int = L.KM_KERNEL_MATERN32


@dataclass
class KernelMatrix:
    """Lazy kernel matrix (src/structstypes.jl:2-23).  pts is an (n, 2) float64 array."""
    x1: np.ndarray
    x2: np.ndarray
    parms: np.ndarray
    kernel: object

    def __init__(self, x1, x2, parms, kernel):
        self.x1 = np.ascontiguousarray(x1, dtype=np.float64)
        self.x2 = np.ascontiguousarray(x2, dtype=np.float64)
        self.parms = np.ascontiguousarray(parms, dtype=np.float64)
        self.kernel = kernel
        if self.x1.ndim != 2 or self.x1.shape[1] != 2 or self.x2.ndim != 2 or self.x2.shape[1] != 2:
            raise KMError(L.KM_ERR_BAD_ARG, "points must be (n, 2) arrays")

    @property
    def shape(self):
        return (len(self.x1), len(self.x2))


# ---- partition --------------------------------------------------------------------------------

def HODLRindices(n: int, lvl):
    """``HODLRindices`` (src/HODLR/src/indices.jl:55-65) through the C ABI: (levels, leaf
    ranges, non-leaf ranges per level), 1-based inclusive like the reference."""
    lib = L.load()
    kind, lv = _level(lvl)
    levels, nleaf, nnon = C.c_int64(), C.c_int64(), C.c_int64()
    _check(None, lib.km_partition_sizes(n, kind, lv, C.byref(levels), C.byref(nleaf), C.byref(nnon)))
    leaf = np.zeros(4 * nleaf.value, dtype=np.int64)
    non = np.zeros(max(4 * nnon.value, 1), dtype=np.int64)
    _check(None, lib.km_partition(n, kind, lv, C.byref(levels), _ip(leaf), _ip(non)))
    leaves = [tuple(int(v) for v in leaf[4 * j:4 * j + 4]) for j in range(nleaf.value)]
    nonleaf, q = [], 0
    for l in range(1, levels.value + 1):
        cnt = nleaf.value >> l
        nonleaf.append([tuple(int(v) for v in non[4 * (q + k):4 * (q + k) + 4]) for k in range(cnt)])
        q += cnt
    if not nonleaf:
        nonleaf = [[]]
    return levels.value, leaves, nonleaf


def nystrom_landmarks(n: int, rank: int) -> np.ndarray:
    """1-based landmark indices ``Int64.(round.(LinRange(1, n, rank)))`` (constructor.jl:31)."""
    lib = L.load()
    out = np.zeros(rank, dtype=np.int64)
    _check(None, lib.km_nystrom_landmarks(n, rank, _ip(out)))
    return out


# ---- HODLR ------------------------------------------------------------------------------------

class _FactorView:
    """``K.W`` / ``K.W'``: products and solves with the symmetric factor."""

    def __init__(self, hk: "KernelHODLR", transpose: bool):
        self._hk = hk
        self._t = transpose

    @property
    def T(self) -> "_FactorView":
        return _FactorView(self._hk, not self._t)

    def ldiv(self, v: np.ndarray) -> np.ndarray:
        """``ldiv!(t, K.W, v)`` / ``ldiv!(t, K.W', v)`` (baseoverloads.jl:126-150)."""
        return self._hk._apply("km_factor_solve", v, self._t)

    def __matmul__(self, v: np.ndarray) -> np.ndarray:
        """``mul!(t, K.W, v)`` / ``mul!(t, K.W', v)`` (baseoverloads.jl:95-124)."""
        return self._hk._apply("km_factor_mul", v, self._t)


class KernelHODLR:
    """``HODLR.KernelHODLR`` held on the GPU (src/HODLR/src/constructor.jl:6-58)."""

    def __init__(self, K: KernelMatrix, ep: float, maxrank: int, lvl, nystrom: bool = False,
                 plel: bool = False, sorted: bool = False, device: int = 0,
                 precision: int = L.KM_PREC_FP64, refine_max_iter: int = 0, refine_tol: float = 1e-10):
        lib = L.load()
        if K.x1.shape != K.x2.shape or not np.array_equal(K.x1, K.x2):
            raise KMError(L.KM_ERR_BAD_ARG, "This function builds symmetric matrices. If you want a non-symmetric "
                          "HODLR matrix, please use the recursive RKernelHODLR, which will only allow matvecs.")
        kid = getattr(K.kernel, "kid", K.kernel)
        cfg = L.KmConfig(device=device, precision=precision, hbm_budget_fraction=0.8,
                         refine_max_iter=refine_max_iter, refine_tol=refine_tol)
        h = C.c_void_p()
        rc = lib.km_create(C.byref(cfg), C.byref(h))
        if rc != L.KM_OK:
            raise KMError(rc, "km_create failed (no CUDA device?)")
        self._h = h
        self.n = K.shape[0]
        self.nys = bool(nystrom)
        self.mrnk = int(maxrank)
        self.ep = float(ep)
        kind, lv = _level(lvl)
        method = L.KM_METHOD_NYSTROM if nystrom else L.KM_METHOD_ACA
        _check(h, lib.km_assemble(h, _dp(K.x1), self.n, int(kid), _dp(K.parms), len(K.parms),
                                  method, float(ep), int(maxrank), kind, int(lv)))
        self.lvl, self.leafindices, self.nonleafindices = HODLRindices(self.n, lvl)
        self.factorized = False

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            L.load().km_destroy(h)
            self._h = None

    # -- helpers --
    def _apply(self, name: str, v: np.ndarray, transpose: Optional[bool] = None) -> np.ndarray:
        lib = L.load()
        vec = np.asarray(v, dtype=np.float64)
        if vec.shape[0] != self.n:
            raise KMError(L.KM_ERR_BAD_ARG, "Matrix and Vector sizes do not agree.")
        b = np.asfortranarray(vec.reshape(self.n, -1))
        out = np.empty_like(b, order="F")
        k = b.shape[1]
        fn = getattr(lib, name)
        if transpose is None:
            rc = fn(self._h, _dp(b), _dp(out), k)
        else:
            rc = fn(self._h, int(transpose), _dp(b), _dp(out), k)
        _check(self._h, rc)
        return out.reshape(vec.shape)

    @property
    def W(self) -> _FactorView:
        return _FactorView(self, False)

    def stats(self) -> L.KmStats:
        st = L.KmStats()
        _check(self._h, L.load().km_get_stats(self._h, C.byref(st)))
        return st

    def block_ranks(self) -> np.ndarray:
        cnt = sum(len(x) for x in self.nonleafindices)
        out = np.zeros(max(cnt, 1), dtype=np.int64)
        _check(self._h, L.load().km_block_ranks(self._h, _ip(out)))
        return out[:cnt]

    def aca_pivots(self, block: int):
        """Row and column pivots (0-based within the block) of ACA block ``block`` (level 1 first)."""
        lib = L.load()
        cap = max(int(self.block_ranks()[block]), 1)
        rows = np.zeros(cap, dtype=np.int64)
        cols = np.zeros(cap, dtype=np.int64)
        rk = C.c_int64()
        _check(self._h, lib.km_aca_pivots(self._h, int(block), cap, _ip(rows), _ip(cols), C.byref(rk)))
        return rows[:rk.value], cols[:rk.value]

    def block_factors(self, block: int):
        """(U, V) of block ``block`` as ``KernelHODLR.U[l][k]``, ``.V[l][k]`` hold them before
        factorisation (structstypes.jl:52-63)."""
        lib = L.load()
        flat = [x for lv in self.nonleafindices for x in lv]
        a, b, c, d = flat[block]
        rk = int(self.block_ranks()[block])
        U = np.zeros((b - a + 1, rk), order="F")
        V = np.zeros((d - c + 1, rk), order="F")
        _check(self._h, lib.km_block_factors(self._h, int(block), _dp(U), _dp(V)))
        return U, V

    # -- reference operations --
    def __matmul__(self, x: np.ndarray) -> np.ndarray:
        """``mul!(target, K::KernelHODLR, src)`` (baseoverloads.jl:152-179)."""
        return self._apply("km_matvec", x)

    def ldiv(self, b: np.ndarray) -> np.ndarray:
        """``K \\ b`` (baseoverloads.jl:181-192, 252-263)."""
        return self._apply("km_solve", b)

    def logdet(self) -> float:
        """``logdet(K)`` (baseoverloads.jl:194-209)."""
        out = C.c_double()
        _check(self._h, L.load().km_logdet(self._h, C.byref(out)))
        return out.value

    def derivative_matvec(self, param: int, x: np.ndarray) -> np.ndarray:
        """``DerivativeHODLR(K, dfun, HK) * x`` for the derivative in parameter ``param``
        (0 scale, 1 range, 2 nugget) (constructor.jl:66-95, baseoverloads.jl:216-234)."""
        lib = L.load()
        vec = np.asarray(x, dtype=np.float64)
        b = np.asfortranarray(vec.reshape(self.n, -1))
        out = np.empty_like(b, order="F")
        _check(self._h, lib.km_derivative_matvec(self._h, int(param), _dp(b), _dp(out), b.shape[1]))
        return out.reshape(vec.shape)

    def nll_grad(self, dat: np.ndarray, vecs=None, profile: bool = False):
        """(NLL, stochastic gradient or None): ``negloglik`` (maxlikfunctions.jl:2-9) and
        ``stoch_gradient`` with shuffle = false (stochasticgradient.jl:30-44); with ``profile``
        ``profile_negloglik`` (maxlikfunctions.jl:11-19) and ``stoch_profile_gradient``
        (stochasticgradient.jl:48-86)."""
        lib = L.load()
        fn = lib.km_profile_nll_grad if profile else lib.km_nll_grad
        y = np.ascontiguousarray(dat, dtype=np.float64).reshape(-1)
        nll = C.c_double()
        if vecs is None:
            _check(self._h, fn(self._h, _dp(y), None, 0, C.byref(nll), None))
            return nll.value, None
        V = np.asfortranarray(np.column_stack(vecs) if isinstance(vecs, (list, tuple)) else vecs,
                              dtype=np.float64)
        g = np.zeros(3)
        _check(self._h, fn(self._h, _dp(y), _dp(V), V.shape[1], C.byref(nll), _dp(g)))
        return nll.value, g

    def nll_grad_seeded(self, dat: np.ndarray, nprobe: int, seed: int, profile: bool = False):
        """``nll_grad`` with ``nprobe`` Rademacher probes drawn on the device: entry (i, j) is +1
        when the top bit of SplitMix64(SplitMix64(seed) + j*n + i) is set, else -1 (stands in
        for ``givesaa(n, m; seed)``, src/utils.jl:22-27)."""
        lib = L.load()
        fn = lib.km_profile_nll_grad_seeded if profile else lib.km_nll_grad_seeded
        y = np.ascontiguousarray(dat, dtype=np.float64).reshape(-1)
        nll = C.c_double()
        g = np.zeros(3)
        _check(self._h, fn(self._h, _dp(y), int(nprobe), int(seed), C.byref(nll), _dp(g) if nprobe > 0 else None))
        return nll.value, (g if nprobe > 0 else None)


def _grad_fisher(HK: "KernelHODLR", dat: np.ndarray, vecs=None, nprobe: int = 0, seed: int = 0):
    lib = L.load()
    y = np.ascontiguousarray(dat, dtype=np.float64).reshape(-1)
    nll = C.c_double()
    g = np.zeros(3)
    F = np.zeros((3, 3), order="F")
    if vecs is None:
        _check(HK._h, lib.km_grad_fisher_seeded(HK._h, _dp(y), int(nprobe), int(seed), C.byref(nll), _dp(g), _dp(F)))
    else:
        V = np.asfortranarray(np.column_stack(vecs) if isinstance(vecs, (list, tuple)) else vecs, dtype=np.float64)
        _check(HK._h, lib.km_grad_fisher(HK._h, _dp(y), _dp(V), V.shape[1], C.byref(nll), _dp(g), _dp(F)))
    return nll.value, g, F


def symmetricfactorize(K: KernelHODLR) -> None:
    """``symmetricfactorize!`` (src/HODLR/src/symfact.jl:6-49)."""
    _check(K._h, L.load().km_factorize(K._h))
    K.factorized = True


def factorize_solve(K: KernelHODLR, b: np.ndarray) -> np.ndarray:
    """``symmetricfactorize!(K)`` followed by ``K \\ b`` (symfact.jl:6-49, baseoverloads.jl:181-192)
    in one call (``km_factorize_solve``: the forward half of the solve overlaps the factorisation);
    the same factor and solution as the two calls."""
    x = K._apply("km_factorize_solve", b)
    K.factorized = True
    return x


def logdet(K: KernelHODLR) -> float:
    return K.logdet()


def negloglik(HK: KernelHODLR, dat: np.ndarray) -> float:
    """``negloglik(HK, dat)`` (src/HODLR/src/maxlikfunctions.jl:2-9)."""
    if not HK.factorized:
        raise KMError(L.KM_ERR_STATE, "The HODLR matrix needs to be factorized for this.")
    return HK.nll_grad(dat)[0]


def stoch_gradient(HK: KernelHODLR, dat: np.ndarray, vecs) -> np.ndarray:
    """``stoch_gradient(K, HK, dat, dfuns, vecs)`` (stochasticgradient.jl:30-44) for the three
    kernel parameters; the derivative functions are the kernel's own."""
    if not HK.factorized:
        raise KMError(L.KM_ERR_STATE, "The matrix needs to be factorized for this to work.")
    return HK.nll_grad(dat, vecs)[1]


def nll_objective(prms, grad, pts: np.ndarray, dat: np.ndarray, kernel, rank: int, lvl, saav,
                  device: int = 0) -> float:
    """``nll_objective(prms, grad, data, opts)`` (maxlikfunctions.jl:29-50): Nystrom assembly with
    ep = 0, factorisation, NLL, and the stochastic gradient written into ``grad`` when it has
    entries."""
    K = KernelMatrix(pts, pts, prms, kernel)
    HK = KernelHODLR(K, 0.0, rank, lvl, nystrom=True, sorted=True, device=device)
    symmetricfactorize(HK)
    if grad is not None and len(grad) > 0:
        nll, g = HK.nll_grad(dat, saav)
        grad[:] = g
        return nll
    return HK.nll_grad(dat)[0]


def stoch_fisher(HK: KernelHODLR, vecs) -> np.ndarray:
    """``stoch_fisher(K, HK, DKs, vecs)`` (src/HODLR/src/stochastichessian.jl:91-115) for the three
    kernel parameters: F_jk = 0.5 mean_v (W^-1 dK_j W'^-1 v)'(W^-1 dK_k W'^-1 v)."""
    if not HK.factorized:
        raise KMError(L.KM_ERR_STATE, "The matrix needs to be factorized.")
    return _grad_fisher(HK, np.ones(HK.n), vecs)[2]


def grad_and_fisher(HK: KernelHODLR, dat: np.ndarray, vecs=None, nprobe: int = 0, seed: int = 0):
    """(NLL, gradient, Fisher matrix) from one set of probes on a factorised Nystrom HODLR: the
    per-matrix part of ``grad_and_fisher_matrix`` (stochastichessian.jl:152-181).  Probes are
    ``vecs`` (host) or ``nprobe`` seeded Rademacher probes drawn on the device."""
    if not HK.factorized:
        raise KMError(L.KM_ERR_STATE, "The matrix needs to be factorized.")
    return _grad_fisher(HK, dat, vecs, nprobe, seed)


def _hessian(HK: "KernelHODLR", dat: np.ndarray, vecs=None, nprobe: int = 0, seed: int = 0, profile: bool = False):
    lib = L.load()
    fs = lib.km_stoch_profile_hessian_seeded if profile else lib.km_stoch_hessian_seeded
    fv = lib.km_stoch_profile_hessian if profile else lib.km_stoch_hessian
    y = np.ascontiguousarray(dat, dtype=np.float64).reshape(-1)
    nll = C.c_double()
    g = np.zeros(3)
    H = np.zeros((3, 3), order="F")
    if vecs is None:
        _check(HK._h, fs(HK._h, _dp(y), int(nprobe), int(seed), C.byref(nll), _dp(g), _dp(H)))
    else:
        V = np.asfortranarray(np.column_stack(vecs) if isinstance(vecs, (list, tuple)) else vecs, dtype=np.float64)
        _check(HK._h, fv(HK._h, _dp(y), _dp(V), V.shape[1], C.byref(nll), _dp(g), _dp(H)))
    return nll.value, g, H


def stoch_hessian(HK: KernelHODLR, dat: np.ndarray, vecs=None, nprobe: int = 0, seed: int = 0,
                  profile: bool = False) -> np.ndarray:
    """``stoch_hessian(K, HK, dat, d1funs, d2funs, vecs; profile)`` (src/HODLR/src/
    stochastichessian.jl:117-147, shuffle = false) for the three kernel parameters, with the
    closed-form second derivatives of the built-in kernels as d2funs; ``profile`` takes the
    profile likelihood's solve term (HODLR_p_hess_slv, :15-31).  Probes are ``vecs`` (host) or
    ``nprobe`` seeded Rademacher probes drawn on the device."""
    if not HK.factorized:
        raise KMError(L.KM_ERR_STATE, "The matrix needs to be factorized.")
    return _hessian(HK, dat, vecs, nprobe, seed, profile)[2]


def grad_fisher_hessian(HK: KernelHODLR, dat: np.ndarray, vecs=None, nprobe: int = 0, seed: int = 0,
                        profile: bool = False):
    """(NLL, gradient, stochastic Hessian) from one set of probes (see ``stoch_hessian``; with
    ``profile`` the profile likelihood's NLL and gradient)."""
    if not HK.factorized:
        raise KMError(L.KM_ERR_STATE, "The matrix needs to be factorized.")
    return _hessian(HK, dat, vecs, nprobe, seed, profile)


def nll_hessian(prms, pts: np.ndarray, dat: np.ndarray, kernel, rank: int, lvl, saav, device: int = 0) -> np.ndarray:
    """``nll_hessian(prms, data, opts)`` (src/HODLR/src/maxlikfunctions.jl:101-116): assemble
    (Nystrom, ep = 0), factorise and return the stochastic Hessian over the probes ``saav``
    (``stoch_hessian`` with the built-in kernels' second derivatives)."""
    K = KernelMatrix(pts, pts, prms, kernel)
    HK = KernelHODLR(K, 0.0, rank, lvl, nystrom=True, sorted=True, device=device)
    symmetricfactorize(HK)
    return _hessian(HK, dat, saav)[2]


def nlpl_hessian(prms, pts: np.ndarray, dat: np.ndarray, kernel, rank: int, lvl, saav, device: int = 0) -> np.ndarray:
    """``nlpl_hessian(prms, data, opts)`` (src/HODLR/src/maxlikfunctions.jl:119-136): assemble
    (Nystrom, ep = 0), factorise and return the stochastic Hessian of the negative log profile
    likelihood over the probes ``saav`` (``stoch_hessian`` with ``profile = true``)."""
    K = KernelMatrix(pts, pts, prms, kernel)
    HK = KernelHODLR(K, 0.0, rank, lvl, nystrom=True, sorted=True, device=device)
    symmetricfactorize(HK)
    return _hessian(HK, dat, saav, profile=True)[2]


def grad_and_fisher_matrix(prms, pts: np.ndarray, dat: np.ndarray, kernel, rank: int, lvl, saav,
                           device: int = 0):
    """``grad_and_fisher_matrix(prm, data, opts)`` (stochastichessian.jl:152-181): assemble
    (Nystrom, ep = 0), factorise, and return (gradient, Fisher matrix)."""
    K = KernelMatrix(pts, pts, prms, kernel)
    HK = KernelHODLR(K, 0.0, rank, lvl, nystrom=True, sorted=True, device=device)
    symmetricfactorize(HK)
    _, g, F = _grad_fisher(HK, dat, saav)
    return g, F


def profile_negloglik(HK: KernelHODLR, dat: np.ndarray) -> float:
    """``profile_negloglik(HK, dat)`` (src/HODLR/src/maxlikfunctions.jl:11-19):
    0.5*(logdet HK + n*log(dat' HK^-1 dat))."""
    if not HK.factorized:
        raise KMError(L.KM_ERR_STATE, "The HODLR matrix needs to be factorized for this.")
    return HK.nll_grad(dat, profile=True)[0]


def stoch_profile_gradient(HK: KernelHODLR, dat: np.ndarray, vecs) -> np.ndarray:
    """``stoch_profile_gradient(K, HK, dat, dfuns, vecs)`` (stochasticgradient.jl:68-86)."""
    if not HK.factorized:
        raise KMError(L.KM_ERR_STATE, "The matrix needs to be factorized for this to work.")
    return HK.nll_grad(dat, vecs, profile=True)[1]


def nlpl_objective(prms, grad, pts: np.ndarray, dat: np.ndarray, kernel, rank: int, lvl, saav,
                   device: int = 0) -> float:
    """``nlpl_objective(prms, grad, data, opts)`` (maxlikfunctions.jl:61-82): ``nll_objective``
    for the profile likelihood."""
    K = KernelMatrix(pts, pts, prms, kernel)
    HK = KernelHODLR(K, 0.0, rank, lvl, nystrom=True, sorted=True, device=device)
    symmetricfactorize(HK)
    if grad is not None and len(grad) > 0:
        nll, g = HK.nll_grad(dat, saav, profile=True)
        grad[:] = g
        return nll
    return HK.nll_grad(dat, profile=True)[0]


def scaleparm_mle(prms, pts: np.ndarray, dat: np.ndarray, kernel, rank: int, lvl, device: int = 0) -> float:
    """``scaleparm_mle`` / ``nlpl_scale`` (maxlikfunctions.jl:21-27,52-58): the profiled scale
    dat' K^-1 dat / n of a freshly assembled and factorised Nystrom HODLR."""
    K = KernelMatrix(pts, pts, prms, kernel)
    HK = KernelHODLR(K, 0.0, rank, lvl, nystrom=True, sorted=True, device=device)
    symmetricfactorize(HK)
    y = np.ascontiguousarray(dat, dtype=np.float64).reshape(-1)
    return float(np.dot(y, HK.ldiv(y))) / y.size


def gpsimulate(kernel, pts: np.ndarray, parms, rank: int, lvl, z: np.ndarray, device: int = 0) -> np.ndarray:
    """``gpsimulate(kernel, locs, parms, opts)`` HODLR branch (maxlikfunctions.jl:148-172):
    out = W z with W the symmetric factor of the Nystrom HODLR (K ~ W W').  ``z`` is the
    standard-normal input (the reference draws it with ``randn``); points are used in the
    order given (k-d sort them first, as ``kdtreesort=true`` does)."""
    K = KernelMatrix(pts, pts, parms, kernel)
    HK = KernelHODLR(K, 0.0, rank, lvl, nystrom=True, device=device)
    symmetricfactorize(HK)
    return HK.W @ np.asarray(z, dtype=np.float64)


class RKernelHODLR:
    """``RKernelHODLR(K, tol, maxrank, lvl)`` (src/HODLR/src/constructor.jl:130-161) held on the GPU:
    the recursive product-only HODLR of K(x1, x2) with x1 and x2 of any lengths, ACA off-diagonal
    blocks and dense diagonal leaves.  ``R @ x`` is the product of baseoverloads.jl:301-305."""

    def __init__(self, K: KernelMatrix, tol: float, maxrank: int = 0, lvl=None, device: int = 0):
        lib = L.load()
        lvl = LogLevel(7) if lvl is None else lvl
        kind, lv = _level(lvl)
        kid = getattr(K.kernel, "kid", K.kernel)
        cfg = L.KmConfig(device=device, precision=L.KM_PREC_FP64, hbm_budget_fraction=0.8, refine_max_iter=0,
                         refine_tol=0.0)
        r = C.c_void_p()
        rc = lib.km_rhodlr_create(C.byref(cfg), _dp(K.x1), K.x1.shape[0], _dp(K.x2), K.x2.shape[0], int(kid),
                                  _dp(K.parms), len(K.parms), float(tol), int(maxrank), kind, int(lv), C.byref(r))
        if rc != L.KM_OK:
            raise KMError(rc, lib.km_rhodlr_create_error().decode())
        self._r = r
        self.shape = (K.x1.shape[0], K.x2.shape[0])
        nb, nl, lvs = C.c_int64(), C.c_int64(), C.c_int64()
        lib.km_rhodlr_info(r, C.byref(nb), C.byref(nl), C.byref(lvs))
        self.nblocks, self.nleaves, self.levels = nb.value, nl.value, lvs.value

    def __del__(self):
        r = getattr(self, "_r", None)
        if r:
            L.load().km_rhodlr_destroy(r)
            self._r = None

    def block_ranks(self) -> np.ndarray:
        out = np.zeros(max(self.nblocks, 1), dtype=np.int64)
        L.load().km_rhodlr_block_ranks(self._r, out.ctypes.data_as(C.POINTER(C.c_int64)))
        return out[:self.nblocks]

    def aca_pivots(self, block: int):
        lib = L.load()
        cap = 8192
        rows = np.zeros(cap, dtype=np.int64)
        cols = np.zeros(cap, dtype=np.int64)
        rk = C.c_int64()
        rc = lib.km_rhodlr_aca_pivots(self._r, int(block), cap, rows.ctypes.data_as(C.POINTER(C.c_int64)),
                                      cols.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(rk))
        if rc != L.KM_OK:
            raise KMError(rc, lib.km_rhodlr_last_error(self._r).decode())
        return rows[:rk.value], cols[:rk.value]

    def __matmul__(self, x: np.ndarray) -> np.ndarray:
        lib = L.load()
        v = np.asarray(x, dtype=np.float64)
        X = np.asfortranarray(v.reshape(self.shape[1], -1))
        Y = np.empty((self.shape[0], X.shape[1]), order="F")
        rc = lib.km_rhodlr_matvec(self._r, _dp(X), _dp(Y), X.shape[1])
        if rc != L.KM_OK:
            raise KMError(rc, lib.km_rhodlr_last_error(self._r).decode())
        return Y.reshape(self.shape[0]) if v.ndim == 1 else Y


class _Scratch:
    """A handle without a problem, for calls that only need a device and a stream."""

    def __init__(self, device: int = 0):
        lib = L.load()
        cfg = L.KmConfig(device=device, precision=L.KM_PREC_FP64, hbm_budget_fraction=0.8, refine_max_iter=0,
                         refine_tol=0.0)
        h = C.c_void_p()
        rc = lib.km_create(C.byref(cfg), C.byref(h))
        if rc != L.KM_OK:
            raise KMError(rc, "km_create failed (no CUDA device?)")
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            L.load().km_destroy(self._h)
            self._h = None


def kd_order(pts: np.ndarray, leaf: int = 32, device: int = 0) -> np.ndarray:
    """k-d ordering permutation of (n, 2) points computed on the GPU (``km_kd_order``): ranges of
    more than ``leaf`` points are sorted stably on their coordinate of larger spread and split at
    floor(len/2), recursively.  Stands in for ``NearestNeighbors.KDTree(pts).data``
    (src/HODLR/src/constructor.jl:180), whose own permutation is not reproduced."""
    P = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 2)
    n = P.shape[0]
    perm = np.empty(n, dtype=np.int64)
    s = _Scratch(device)
    _check(s._h, L.load().km_kd_order(s._h, _dp(P), n, int(leaf), perm.ctypes.data_as(C.POINTER(C.c_int64))))
    return perm


def maxlikdata(pts: np.ndarray, data: np.ndarray, sortmethod: str = "kdtree", leaf: int = 32, device: int = 0):
    """``maxlikdata(pts=, data=, sortmethod=)`` (src/HODLR/src/constructor.jl:171-202): returns the
    (points, data) pair sorted by the GPU k-d ordering (``"kdtree"``) or unchanged
    (``"nothing"``); any other method raises as the reference does.  Each datum travels with its
    own point (the reference's data_reorder looks data up by point value, src/utils.jl:22-25)."""
    P = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 2)
    y = np.ascontiguousarray(data, dtype=np.float64).reshape(-1)
    if P.shape[0] != y.size:
        raise KMError(L.KM_ERR_BAD_ARG, "points and data disagree in length")
    m = str(sortmethod).lower().lstrip(":")
    if m == "nothing":
        return P.copy(), y.copy()
    if m != "kdtree":
        raise KMError(L.KM_ERR_BAD_ARG, "The options are :Nothing and :KDTree")
    n = P.shape[0]
    ps = np.empty_like(P)
    ys = np.empty_like(y)
    s = _Scratch(device)
    _check(s._h, L.load().km_maxlikdata(s._h, _dp(P), _dp(y), n, int(leaf), _dp(ps), _dp(ys), None))
    return ps, ys


def probe_fp32_tflops(device: int = 0) -> float:
    out = C.c_double()
    rc = L.load().km_probe_fp32_tflops(device, C.byref(out))
    if rc != L.KM_OK:
        raise KMError(rc, "FP32 probe failed")
    return out.value


def probe_fp64_tflops(device: int = 0) -> float:
    out = C.c_double()
    rc = L.load().km_probe_fp64_tflops(device, C.byref(out))
    if rc != L.KM_OK:
        raise KMError(rc, "FP64 probe failed")
    return out.value
