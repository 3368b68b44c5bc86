"""ctypes binding of libkmhodlr.so (declarations in include/kmhodlr.h).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libkmhodlr.so"

KM_OK = 0
KM_ERR_BAD_ARG = 1
KM_ERR_NOT_SPD = 2
KM_ERR_OOM = 3
KM_ERR_CUDA = 4
KM_ERR_STATE = 5
KM_ERR_TIMEOUT = 6
KM_ERR_UNSUPPORTED = 7
KM_ERR_ACA = 8

KM_KERNEL_RATQUAD = 0
KM_KERNEL_MATERN32 = 1
KM_LEVEL_FIXED = 0
KM_LEVEL_LOG = 1
KM_METHOD_ACA = 0
KM_METHOD_NYSTROM = 1
KM_PREC_FP64 = 0
KM_PREC_MIXED = 1

PROF_CLASSES = ["eval", "leaf_chol", "leaf_tri", "leaf_qr", "node", "sweep", "leaf_refl", "leaf_apply",
                "other", "aca", "leaf_tc"]


class KmConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("hbm_budget_fraction", C.c_double),
                ("refine_max_iter", C.c_int), ("refine_tol", C.c_double)]


class KmStats(C.Structure):
    _fields_ = [("assemble_ms", C.c_double), ("factorize_ms", C.c_double), ("solve_ms", C.c_double),
                ("matvec_ms", C.c_double), ("logdet_ms", C.c_double), ("grad_ms", C.c_double),
                ("device_bytes", C.c_int64), ("kernel_launches", C.c_int64),
                ("refine_iterations", C.c_int), ("refine_residual", C.c_double),
                ("precision_fallbacks", C.c_int64)]


KM_REQ_NLL_GRAD = 0
KM_REQ_FACTOR = 1
KM_REQ_SOLVE = 2
KM_REQ_RELEASE = 3
KM_REQ_PROFILE_NLL_GRAD = 4


class KmProblem(C.Structure):
    _fields_ = [("n", C.c_int64), ("pts", C.POINTER(C.c_double)), ("y", C.POINTER(C.c_double)),
                ("params", C.c_double * 3)]


class KmBatchOpts(C.Structure):
    _fields_ = [("kernel_id", C.c_int), ("rank", C.c_int64), ("level_kind", C.c_int), ("level", C.c_int64),
                ("nprobe", C.c_int64), ("probe_seed", C.c_uint64), ("profile", C.c_int)]


class KmRequest(C.Structure):
    _fields_ = [("kind", C.c_int), ("prob", KmProblem), ("nprobe", C.c_int64), ("probe_seed", C.c_uint64),
                ("factor_id", C.c_int64), ("b", C.POINTER(C.c_double)), ("x", C.POINTER(C.c_double)),
                ("nrhs", C.c_int64)]


class KmResult(C.Structure):
    _fields_ = [("status", C.c_int), ("nll", C.c_double), ("grad", C.c_double * 3), ("logdet", C.c_double),
                ("factor_id", C.c_int64), ("queue_ms", C.c_double), ("run_ms", C.c_double)]


class KmServeOpts(C.Structure):
    _fields_ = [("kernel_id", C.c_int), ("rank", C.c_int64), ("level_kind", C.c_int), ("level", C.c_int64),
                ("nworkers", C.c_int)]


class KmServeStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("rejected", C.c_int64), ("resident_factors", C.c_int64), ("bytes_in_use", C.c_int64),
                ("peak_bytes", C.c_int64), ("budget_bytes", C.c_int64), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("mean_ms", C.c_double)]


_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int64)
_H = C.c_void_p

# name -> (restype, argtypes); every symbol declared in include/kmhodlr.h
SIGNATURES = {
    "km_partition_sizes": (C.c_int, [C.c_int64, C.c_int, C.c_int64, _IP, _IP, _IP]),
    "km_partition": (C.c_int, [C.c_int64, C.c_int, C.c_int64, _IP, _IP, _IP]),
    "km_nystrom_landmarks": (C.c_int, [C.c_int64, C.c_int64, _IP]),
    "km_create": (C.c_int, [C.POINTER(KmConfig), C.POINTER(_H)]),
    "km_destroy": (C.c_int, [_H]),
    "km_last_error": (C.c_char_p, [_H]),
    "km_get_stats": (C.c_int, [_H, C.POINTER(KmStats)]),
    "km_assemble": (C.c_int, [_H, _DP, C.c_int64, C.c_int, _DP, C.c_int, C.c_int, C.c_double, C.c_int64,
                              C.c_int, C.c_int64]),
    "km_block_ranks": (C.c_int, [_H, _IP]),
    "km_aca_pivots": (C.c_int, [_H, C.c_int64, C.c_int64, _IP, _IP, _IP]),
    "km_block_factors": (C.c_int, [_H, C.c_int64, _DP, _DP]),
    "km_matvec": (C.c_int, [_H, _DP, _DP, C.c_int64]),
    "km_factorize": (C.c_int, [_H]),
    "km_solve": (C.c_int, [_H, _DP, _DP, C.c_int64]),
    "km_factor_solve": (C.c_int, [_H, C.c_int, _DP, _DP, C.c_int64]),
    "km_factor_mul": (C.c_int, [_H, C.c_int, _DP, _DP, C.c_int64]),
    "km_logdet": (C.c_int, [_H, _DP]),
    "km_matvec_dev": (C.c_int, [_H, _P, _P, C.c_int64]),
    "km_solve_dev": (C.c_int, [_H, _P, _P, C.c_int64]),
    "km_factorize_solve": (C.c_int, [_H, _DP, _DP, C.c_int64]),
    "km_factorize_solve_dev": (C.c_int, [_H, _P, _P, C.c_int64]),
    "km_factor_solve_dev": (C.c_int, [_H, C.c_int, _P, _P, C.c_int64]),
    "km_factor_mul_dev": (C.c_int, [_H, C.c_int, _P, _P, C.c_int64]),
    "km_derivative_matvec": (C.c_int, [_H, C.c_int, _DP, _DP, C.c_int64]),
    "km_nll_grad": (C.c_int, [_H, _DP, _DP, C.c_int64, _DP, _DP]),
    "km_probe_fp64_tflops": (C.c_int, [C.c_int, _DP]),
    "km_probe_fp32_tflops": (C.c_int, [C.c_int, _DP]),
    "km_probe_tc_gemm": (C.c_int, [C.c_int, _DP, _DP, C.c_int, _DP]),
    "km_set_wait_limit": (C.c_int, [_H, C.c_int64]),
    "km_assemble_dev": (C.c_int, [_H, _P, C.c_int64, C.c_int, _DP, C.c_int, C.c_int, C.c_double, C.c_int64,
                                  C.c_int, C.c_int64]),
    "km_set_stream": (C.c_int, [_H, _P]),
    "km_profile_enable": (C.c_int, [_H, C.c_int]),
    "km_profile_get": (C.c_int, [_H, C.c_int, _DP, _IP]),
    "km_solve_noalloc": (C.c_int, [_H, _P, _P, C.c_int64]),
    "km_nll_grad_seeded": (C.c_int, [_H, _DP, C.c_int64, C.c_uint64, _DP, _DP]),
    "km_profile_nll_grad": (C.c_int, [_H, _DP, _DP, C.c_int64, _DP, _DP]),
    "km_grad_fisher": (C.c_int, [_H, _DP, _DP, C.c_int64, _DP, _DP, _DP]),
    "km_kd_order": (C.c_int, [_H, _DP, C.c_int64, C.c_int64, C.POINTER(C.c_int64)]),
    "km_rhodlr_create": (C.c_int, [C.POINTER(KmConfig), _DP, C.c_int64, _DP, C.c_int64, C.c_int, _DP, C.c_int,
                                   C.c_double, C.c_int64, C.c_int, C.c_int64, C.POINTER(_P)]),
    "km_rhodlr_destroy": (C.c_int, [_P]),
    "km_rhodlr_create_error": (C.c_char_p, []),
    "km_rhodlr_last_error": (C.c_char_p, [_P]),
    "km_rhodlr_info": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "km_rhodlr_block_ranks": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "km_rhodlr_aca_pivots": (C.c_int, [_P, C.c_int64, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int64)]),
    "km_rhodlr_matvec": (C.c_int, [_P, _DP, _DP, C.c_int64]),
    "km_maxlikdata": (C.c_int, [_H, _DP, _DP, C.c_int64, C.c_int64, _DP, _DP, C.POINTER(C.c_int64)]),
    "km_grad_fisher_seeded": (C.c_int, [_H, _DP, C.c_int64, C.c_uint64, _DP, _DP, _DP]),
    "km_stoch_hessian": (C.c_int, [_H, _DP, _DP, C.c_int64, _DP, _DP, _DP]),
    "km_stoch_hessian_seeded": (C.c_int, [_H, _DP, C.c_int64, C.c_uint64, _DP, _DP, _DP]),
    "km_stoch_profile_hessian": (C.c_int, [_H, _DP, _DP, C.c_int64, _DP, _DP, _DP]),
    "km_stoch_profile_hessian_seeded": (C.c_int, [_H, _DP, C.c_int64, C.c_uint64, _DP, _DP, _DP]),
    "km_profile_nll_grad_seeded": (C.c_int, [_H, _DP, C.c_int64, C.c_uint64, _DP, _DP]),
    "km_trim": (C.c_int, [_H]),
    "km_estimate_bytes": (C.c_int64, [C.c_int64, C.c_int64, C.c_int, C.c_int64, C.c_int64, C.c_int]),
    "km_batch_create": (C.c_int, [C.POINTER(KmConfig), C.c_int, C.POINTER(_P)]),
    "km_batch_destroy": (C.c_int, [_P]),
    "km_batch_nll_grad": (C.c_int, [_P, C.POINTER(KmBatchOpts), C.c_int64, C.POINTER(KmProblem), _DP, _DP,
                                    C.POINTER(C.c_int)]),
    "km_batch_last_error": (C.c_char_p, [_P]),
    "km_serve_create": (C.c_int, [C.POINTER(KmConfig), C.POINTER(KmServeOpts), C.POINTER(_P)]),
    "km_serve_submit": (C.c_int, [_P, C.POINTER(KmRequest), C.POINTER(C.c_uint64)]),
    "km_serve_wait": (C.c_int, [_P, C.c_uint64, C.c_int64, C.POINTER(KmResult)]),
    "km_serve_stats_get": (C.c_int, [_P, C.POINTER(KmServeStats)]),
    "km_serve_destroy": (C.c_int, [_P]),
}

_lib = None


def load() -> C.CDLL:
    """Load libkmhodlr.so (built by kmhodlr.build) and declare every exported symbol."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: run kmhodlr.build.build() (no CPU fallback exists)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
