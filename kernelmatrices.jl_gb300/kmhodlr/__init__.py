"""kmhodlr: GB300 HODLR engine for the KernelMatrices.jl hot path (Python mirror of the API).

The compute runs in libkmhodlr.so (hand-written sm_103a CUDA kernels behind a C ABI,
include/kmhodlr.h).  Importing this package does not require a GPU; creating a KernelHODLR does.
"""
from ._lib import load, LIB_PATH, KM_PREC_FP64, KM_PREC_MIXED  # noqa: F401
from .hodlr import (  # noqa: F401
    FixedLevel, LogLevel, KernelMatrix, KernelHODLR, RatQuad, Matern32, HODLRindices,
    KMError, PosDefException, symmetricfactorize, factorize_solve, logdet, nystrom_landmarks, probe_fp64_tflops,
    probe_fp32_tflops,
    negloglik, stoch_gradient, nll_objective, profile_negloglik, stoch_profile_gradient, nlpl_objective,
    scaleparm_mle, gpsimulate, stoch_fisher, grad_and_fisher, grad_and_fisher_matrix, stoch_hessian,
    grad_fisher_hessian, nll_hessian, nlpl_hessian, kd_order, maxlikdata,
    RKernelHODLR,
)
from .serving import BatchEngine, Server, Problem, Result, estimate_bytes  # noqa: F401
