"""Tensor-core leaf stage of the mixed form (km_leaf_tc.cu).

* The tensor cores' data layout: single-slice integer products (|v| <= 128, 64 terms) must equal
  the exact integer product, the largest sums included.
* The split product of one tile (float-pair inputs cut into 7 bf16 slices, 28 slice products
  summed per diagonal in fp32, diagonals added in float pairs) against the exact product of the
  same float-pair inputs: within 2^-40 of (row max x column max), rows of very different scales
  and a zero row included.
* The blocked augmented leaf Cholesky inside the mixed factorisation: logdet within 1e-6 and
  solves within 1e-8 of the FP64 form on leaves of 256, 312/313 and 375 points (full and partial
  64-column blocks) with ranks 72, 80 and 40, and the same results as the float-pair CUDA-core
  leaf kernels (KM_LEAF_TC=0, run in a child process) to 1e-9.
"""
import ctypes as C
import json
import math
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def _probe(lib, A, B, mode):
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    out = np.zeros((128, 64))
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    rc = lib.km_probe_tc_gemm(0, dp(A), dp(B), mode, dp(out))
    assert rc == 0, rc
    return out


def test_single_slice_products_are_exact(lib):
    rng = np.random.default_rng(1)
    A = rng.integers(-128, 129, size=(128, 64))
    B = rng.integers(-128, 129, size=(64, 64))
    assert np.array_equal(_probe(lib, A, B, 0), (A @ B.T).astype(np.float64))
    # the largest sums: every product 2^14
    A = np.full((128, 64), 128.0)
    B = np.full((64, 64), -128.0)
    assert np.all(_probe(lib, A, B, 0) == -64 * 128 * 128)
    # a permutation pattern: C[i, j] = A[i, j] picks out single entries of the layout
    A = rng.integers(-128, 129, size=(128, 64)).astype(np.float64)
    assert np.array_equal(_probe(lib, A, np.eye(64), 0), A)


def _ff(a):
    hi = a.astype(np.float32).astype(np.float64)
    lo = (a - hi).astype(np.float32).astype(np.float64)
    return hi + lo


def _exact_nt(A, B):
    """A B' of doubles rounded once (Dekker splits, exact partial products, math.fsum)."""
    def split(a):
        c = a * 134217729.0
        h = c - (c - a)
        return h, a - h
    Ah, Al = split(A)
    Bh, Bl = split(B)
    out = np.empty((A.shape[0], B.shape[0]))
    for i in range(A.shape[0]):
        parts = np.concatenate([Ah[i] * Bh, Ah[i] * Bl, Al[i] * Bh, Al[i] * Bl], axis=1)
        for j in range(B.shape[0]):
            out[i, j] = math.fsum(parts[j])
    return out


def test_split_product_accuracy(lib):
    rng = np.random.default_rng(2)
    A = rng.standard_normal((128, 64)) * np.exp2(rng.integers(-20, 21, size=(128, 1)))
    B = rng.standard_normal((64, 64)) * np.exp2(rng.integers(-10, 11, size=(64, 1)))
    A[5] = 0.0
    A[7, ::2] *= 1e-9          # one row with entries nine orders apart
    B[3, 1:] = 1e-12           # one row dominated by a single entry
    Af, Bf = _ff(A), _ff(B)
    got = _probe(lib, A, B, 1)
    ref = _exact_nt(Af, Bf)
    scale = np.outer(np.abs(Af).max(axis=1), np.abs(Bf).max(axis=1))
    assert np.all(got[5] == 0.0)
    assert np.all(np.abs(got - ref) <= 2.0 ** -40 * scale), np.max(np.abs(got - ref) / np.maximum(scale, 1e-300))


CASES = [  # n, level, rank: leaf sizes 256 (r 72), 312/313 (r 80), 375 (r 40)
    (16384, 6, 72),
    (5000, 4, 80),
    (6000, 4, 40),
]


def _results(n, level, rank, mixed):
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    pts = uniform_points(n, 41)
    rhs = np.random.default_rng(42).standard_normal((n, 4))
    prec = K.KM_PREC_MIXED if mixed else K.KM_PREC_FP64
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, [1.0, 0.1, 1e-3], K.Matern32()), 0.0, rank, K.FixedLevel(level),
                       nystrom=True, precision=prec)
    K.symmetricfactorize(hk)
    return hk.logdet(), hk.ldiv(rhs), hk.stats().precision_fallbacks


@pytest.mark.parametrize("n,level,rank", CASES)
def test_leaf_tc_factorisation_matches_fp64(lib, n, level, rank):
    ld64, x64, _ = _results(n, level, rank, False)
    ldm, xm, fb = _results(n, level, rank, True)
    assert fb == 0
    assert abs(ldm - ld64) < 1e-6
    assert np.linalg.norm(xm - x64) / np.linalg.norm(x64) < 1e-8


def test_leaf_tc_matches_cuda_core_leaf_kernels(lib):
    """The tensor-core leaf stage against the float-pair CUDA-core leaf kernels on the same input."""
    code = (
        "import json, sys\n"
        f"sys.path[:0] = [{str(ROOT)!r}, {str(ROOT / 'kernelmatrices.jl_gb300')!r}, {str(ROOT / 'tests')!r}]\n"
        "from test_gpu_tc import _results\n"
        "out = {}\n"
        f"for n, lv, rk in {CASES!r}:\n"
        "    ld, x, fb = _results(n, lv, rk, True)\n"
        "    out[str(n)] = [ld, x.tolist()]\n"
        "print(json.dumps(out))\n")
    env = dict(os.environ, KM_LEAF_TC="0")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    ref = json.loads(r.stdout.strip().splitlines()[-1])
    for n, lv, rk in CASES:
        ld, x, _ = _results(n, lv, rk, True)
        ld0, x0 = ref[str(n)]
        x0 = np.array(x0)
        assert abs(ld - ld0) < 1e-6
        assert np.linalg.norm(x - x0) / np.linalg.norm(x0) < 1e-9


def test_second_factorisation_of_one_assembly(lib):
    """A second symmetricfactorize! of the same assembly starts again from the leaf matrices."""
    import kmhodlr as K
    from kmhodlr.data import uniform_points
    n = 8192
    pts = uniform_points(n, 44)
    rhs = np.random.default_rng(45).standard_normal((n, 2))
    hk = K.KernelHODLR(K.KernelMatrix(pts, pts, [1.0, 0.1, 1e-3], K.Matern32()), 0.0, 72, K.FixedLevel(5),
                       nystrom=True, precision=K.KM_PREC_MIXED)
    K.symmetricfactorize(hk)
    ld1, x1 = hk.logdet(), hk.ldiv(rhs)
    K.symmetricfactorize(hk)
    assert hk.logdet() == ld1
    assert np.array_equal(hk.ldiv(rhs), x1)
