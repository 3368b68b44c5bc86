"""Batched and serving forms of the likelihood path (``km_batch_*`` / ``km_serve_*`` in
include/kmhodlr.h).

``BatchEngine.nll_grad`` evaluates ``nll_objective`` (src/HODLR/src/maxlikfunctions.jl:29-50:
Nystrom assembly, ``symmetricfactorize!``, ``negloglik`` and ``stoch_gradient``) for many
independent datasets at once.  ``Server`` accepts a stream of likelihood, factor, solve and
release requests and runs them with continuous batching under an HBM budget.  Both drive the
same handle code as ``KernelHODLR``.  Probes are drawn on the device from a seed: entry (i, j)
of a problem's n x nprobe block is +1 when the top bit of SplitMix64(SplitMix64(seed) + j*n + i)
is set, else -1.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import _lib as L
from .hodlr import KMError, PosDefException, _level


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _raise(rc: int, msg: str):
    if rc == L.KM_ERR_NOT_SPD:
        raise PosDefException(rc, msg)
    raise KMError(rc, msg)


def estimate_bytes(n: int, rank: int, lvl, ncols: int = 1, with_grad: bool = False) -> int:
    """Device bytes one handle holds for this problem shape (``km_estimate_bytes``)."""
    kind, lv = _level(lvl)
    return int(L.load().km_estimate_bytes(int(n), int(rank), kind, int(lv), int(ncols), int(bool(with_grad))))


@dataclass
class Problem:
    """One dataset: (n, 2) points in the caller's order, n observations, 3 kernel parameters."""
    pts: np.ndarray
    y: np.ndarray
    params: Sequence[float]

    def _c(self, keep: list) -> L.KmProblem:
        pts = np.ascontiguousarray(self.pts, dtype=np.float64).reshape(-1)
        y = np.ascontiguousarray(self.y, dtype=np.float64).reshape(-1)
        if pts.size != 2 * y.size:
            raise KMError(L.KM_ERR_BAD_ARG, "points and observations disagree in length")
        keep += [pts, y]
        p = L.KmProblem()
        p.n = y.size
        p.pts = _dp(pts)
        p.y = _dp(y)
        for i in range(3):
            p.params[i] = float(self.params[i])
        return p


class BatchEngine:
    """A pool of ``nworkers`` GPU handles (own streams and host threads) for independent problems."""

    def __init__(self, nworkers: int = 8, device: int = 0, precision: int = L.KM_PREC_FP64):
        lib = L.load()
        cfg = L.KmConfig(device=device, precision=precision, hbm_budget_fraction=0.8, refine_max_iter=0,
                         refine_tol=0.0)
        b = C.c_void_p()
        rc = lib.km_batch_create(C.byref(cfg), int(nworkers), C.byref(b))
        if rc != L.KM_OK:
            raise KMError(rc, "km_batch_create failed (no CUDA device?)")
        self._b = b

    def close(self):
        if getattr(self, "_b", None):
            L.load().km_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        self.close()

    def nll_grad(self, problems: List[Problem], kernel, rank: int, lvl, nprobe: int = 72, seed: int = 0,
                 raise_on_error: bool = True, profile: bool = False):
        """(nll[nprob], grad[nprob, 3] or None, status[nprob]); problem b uses probe seed seed + b.
        ``profile`` evaluates the profile likelihood (``nlpl_objective``) instead."""
        lib = L.load()
        kind, lv = _level(lvl)
        o = L.KmBatchOpts(kernel_id=int(getattr(kernel, "kid", kernel)), rank=int(rank), level_kind=kind,
                          level=int(lv), nprobe=int(nprobe), probe_seed=int(seed), profile=int(bool(profile)))
        keep: list = []
        arr = (L.KmProblem * max(len(problems), 1))()
        for i, p in enumerate(problems):
            arr[i] = p._c(keep)
        m = len(problems)
        nll = np.zeros(m)
        grad = np.zeros((m, 3))
        status = np.zeros(m, dtype=np.int32)
        rc = lib.km_batch_nll_grad(self._b, C.byref(o), m, arr, _dp(nll), _dp(grad) if nprobe > 0 else None,
                                   status.ctypes.data_as(C.POINTER(C.c_int)))
        if rc != L.KM_OK and raise_on_error:
            _raise(rc, lib.km_batch_last_error(self._b).decode())
        return nll, (grad if nprobe > 0 else None), status


@dataclass
class Result:
    status: int
    nll: float
    grad: np.ndarray
    logdet: float
    factor_id: int
    queue_ms: float
    run_ms: float
    x: Optional[np.ndarray] = None


class Server:
    """Continuous-batching server (``km_serve_*``).  Inputs passed to ``submit_*`` are kept alive
    by this object until their result has been collected with ``wait``."""

    def __init__(self, kernel, rank: int, lvl, nworkers: int = 8, device: int = 0,
                 precision: int = L.KM_PREC_FP64, hbm_budget_fraction: float = 0.8):
        lib = L.load()
        kind, lv = _level(lvl)
        cfg = L.KmConfig(device=device, precision=precision, hbm_budget_fraction=float(hbm_budget_fraction),
                         refine_max_iter=0, refine_tol=0.0)
        o = L.KmServeOpts(kernel_id=int(getattr(kernel, "kid", kernel)), rank=int(rank), level_kind=kind,
                          level=int(lv), nworkers=int(nworkers))
        s = C.c_void_p()
        rc = lib.km_serve_create(C.byref(cfg), C.byref(o), C.byref(s))
        if rc != L.KM_OK:
            raise KMError(rc, "km_serve_create failed")
        self._s = s
        self._keep = {}

    def _submit(self, req: L.KmRequest, keep) -> int:
        t = C.c_uint64()
        rc = L.load().km_serve_submit(self._s, C.byref(req), C.byref(t))
        if rc != L.KM_OK:
            raise KMError(rc, "km_serve_submit rejected the request")
        self._keep[t.value] = keep
        return t.value

    def submit_nll_grad(self, prob: Problem, nprobe: int = 72, seed: int = 0, profile: bool = False) -> int:
        keep: list = []
        req = L.KmRequest(kind=L.KM_REQ_PROFILE_NLL_GRAD if profile else L.KM_REQ_NLL_GRAD, nprobe=int(nprobe),
                          probe_seed=int(seed))
        req.prob = prob._c(keep)
        return self._submit(req, (keep, None))

    def submit_factor(self, prob: Problem) -> int:
        keep: list = []
        req = L.KmRequest(kind=L.KM_REQ_FACTOR)
        req.prob = prob._c(keep)
        return self._submit(req, (keep, None))

    def submit_solve(self, factor_id: int, b: np.ndarray) -> int:
        B = np.asfortranarray(b, dtype=np.float64)
        nrhs = 1 if B.ndim == 1 else B.shape[1]
        X = np.empty_like(B, order="F")
        req = L.KmRequest(kind=L.KM_REQ_SOLVE, factor_id=int(factor_id), nrhs=nrhs)
        req.b = _dp(B)
        req.x = _dp(X)
        return self._submit(req, ([B], X))

    def submit_release(self, factor_id: int) -> int:
        return self._submit(L.KmRequest(kind=L.KM_REQ_RELEASE, factor_id=int(factor_id)), ([], None))

    def wait(self, ticket: int, timeout_ms: int = -1) -> Result:
        r = L.KmResult()
        rc = L.load().km_serve_wait(self._s, int(ticket), int(timeout_ms), C.byref(r))
        if rc != L.KM_OK:
            raise KMError(rc, "km_serve_wait failed" if rc != L.KM_ERR_TIMEOUT else "request still running")
        keep = self._keep.pop(ticket, ([], None))
        return Result(r.status, r.nll, np.array(r.grad[:]), r.logdet, r.factor_id, r.queue_ms, r.run_ms, keep[1])

    def stats(self) -> L.KmServeStats:
        st = L.KmServeStats()
        L.load().km_serve_stats_get(self._s, C.byref(st))
        return st

    def close(self):
        if getattr(self, "_s", None):
            L.load().km_serve_destroy(self._s)
            self._s = None
            self._keep.clear()

    def __del__(self):
        self.close()

