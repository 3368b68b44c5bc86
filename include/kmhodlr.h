/*
 * kmhodlr.h -- C ABI of the GB300 HODLR engine for the KernelMatrices.jl hot path.
 *
 * Every entry point is a plain C function (extern "C"), takes plain pointers and sizes, and
 * returns an int status (KM_OK == 0).  Arrays are column-major FP64, as Julia stores them.
 * Points are `const double*` holding 2*n values in (x, y) pairs -- the memory layout of a Julia
 * `Vector{SVector{2,Float64}}`, so a Julia caller passes `pointer(pts)` without a copy.
 * Host-pointer entry points copy their inputs to the device and their outputs back; the `_dev`
 * variants take device pointers that stay resident in HBM.
 *
 * Each declaration names the reference interface it replaces (file:line inside the
 * KernelMatrices.jl project).  The reference raises Julia exceptions; here a non-zero status is
 * returned and km_last_error() gives the message.  KM_ERR_NOT_SPD stands for PosDefException.
 *
 * Threading: one CUDA stream per handle; different handles may be used from different threads.
 * A single handle must not be used from two threads at once.
 */
#ifndef KMHODLR_H
#define KMHODLR_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------- */
enum km_status {
  KM_OK = 0,
  KM_ERR_BAD_ARG = 1,      /* invalid argument (sizes, ids, null pointers)                   */
  KM_ERR_NOT_SPD = 2,      /* a Cholesky pivot was <= 0 (Julia PosDefException)              */
  KM_ERR_OOM = 3,          /* device allocation failed or the HBM budget would be exceeded   */
  KM_ERR_CUDA = 4,         /* a CUDA runtime call failed                                      */
  KM_ERR_STATE = 5,        /* call out of order, e.g. solve before factorize                  */
  KM_ERR_TIMEOUT = 6,      /* a bounded device-side wait ran out                               */
  KM_ERR_UNSUPPORTED = 7,  /* valid request this build does not implement                     */
  KM_ERR_ACA = 8           /* ACA failure (reference: "Incompatible maxrank or matrix dims")  */
};

/* ---- enumerations ------------------------------------------------------------------------- */
enum km_kernel_id {
  /* p1^2 / (1 + (r/p2)^2)^2 + p3 * [x == y]          (README.md:42-48 kernelfunction)       */
  KM_KERNEL_RATQUAD = 0,
  /* p1 * (1 + sqrt3 r/p2) exp(-sqrt3 r/p2) + p3*[x==y] (mtn_kernfun at nu = 3/2,
   * src/covariancefunctions.jl:258-266, with mtn_cor's |x| <= 1e-8 -> 1 rule, :209-212)      */
  KM_KERNEL_MATERN32 = 1
};
enum km_level_kind { KM_LEVEL_FIXED = 0, KM_LEVEL_LOG = 1 };  /* FixedLevel / LogLevel         */
enum km_method { KM_METHOD_ACA = 0, KM_METHOD_NYSTROM = 1 };
enum km_precision {
  KM_PREC_FP64 = 0,   /* every step in FP64                                                   */
  KM_PREC_MIXED = 1   /* FP32 bulk factorisation + FP64 refinement of solves                  */
};

typedef struct km_config {
  int device;                  /* CUDA device ordinal                                          */
  int precision;               /* enum km_precision                                             */
  double hbm_budget_fraction;  /* fraction of device memory a handle may hold (0 => 0.8)       */
  int refine_max_iter;         /* mixed precision: max refinement iterations (0 => 30)         */
  double refine_tol;           /* mixed precision: relative residual target (0 => 1e-10)       */
} km_config;

typedef struct km_stats {
  double assemble_ms, factorize_ms, solve_ms, matvec_ms, logdet_ms, grad_ms;  /* last call     */
  int64_t device_bytes;        /* bytes of device memory held by the handle                    */
  int64_t kernel_launches;     /* kernels launched by the handle since creation                 */
  int refine_iterations;       /* iterations used by the last mixed-precision solve             */
  double refine_residual;      /* final relative residual of that solve                         */
  int64_t precision_fallbacks; /* mixed-precision factorisations redone in FP64 after a
                                  non-positive pivot in float-pair arithmetic                  */
} km_stats;

typedef struct km_handle km_handle;

/* ---- tree partition (pure host, bit-exact with the reference) ------------------------------- */

/* Sizes of the HODLR partition of n points: number of levels, leaves and non-leaf blocks.
 * Replaces _leafsizes (src/HODLR/src/indices.jl:5-24).  n must satisfy 1 <= n < 2^48. */
int km_partition_sizes(int64_t n, int level_kind, int64_t level, int64_t* out_levels,
                       int64_t* out_nleaf, int64_t* out_nnonleaf);

/* 1-based inclusive index ranges of every leaf ([s,e,s,e], 4 per leaf) and non-leaf block
 * ([a,b,c,d], 4 per block, level 1 first; rows a:b = second child, cols c:d = first child).
 * Replaces HODLRindices (src/HODLR/src/indices.jl:55-65) with _leafindices (:29-37) and
 * _nextlevel (:40-51).  Buffers sized from km_partition_sizes; either may be NULL. */
int km_partition(int64_t n, int level_kind, int64_t level, int64_t* out_levels,
                 int64_t* leaf, int64_t* nonleaf);

/* Nystrom landmark indices (1-based): Int64.(round.(LinRange(1, n, rank)))
 * (src/HODLR/src/constructor.jl:31). */
int km_nystrom_landmarks(int64_t n, int64_t rank, int64_t* out);

/* ---- handle lifecycle -------------------------------------------------------------------- */
/* A handle holds one problem's device state: it stands for the KernelHODLR object
 * (src/HODLR/src/structstypes.jl:52-63) together with the factor W it keeps after
 * symmetricfactorize! (FactorHODLR, structstypes.jl:46-49).  km_last_error gives the message of
 * the last failing call (where the reference throws, with the reference's message where one
 * exists); km_get_stats has no reference counterpart. */
int km_create(const km_config* cfg, km_handle** out);
int km_destroy(km_handle* h);
const char* km_last_error(const km_handle* h);
int km_get_stats(const km_handle* h, km_stats* out);

/* ---- assembly ---------------------------------------------------------------------------- */

/* Assemble the HODLR matrix of the kernel matrix K[i,j] = k(pts[i], pts[j], params) with
 * nparams == 3 parameters (scale, range, nugget).
 * Replaces KernelMatrix(pts, pts, parms, kernel) (src/structstypes.jl:17) followed by
 * KernelHODLR(K, ep, maxrank, lvl; nystrom) (src/HODLR/src/constructor.jl:6-58):
 *   method KM_METHOD_NYSTROM: nystrom_uvt blocks (src/factorizations.jl:86-94), rank = maxrank;
 *   method KM_METHOD_ACA:     ACA blocks (src/factorizations.jl:9-84) with tolerance tol and
 *                             rank cap maxrank (0 = none). */
int km_assemble(km_handle* h, const double* pts, int64_t n, int kernel_id, const double* params,
                int nparams, int method, double tol, int64_t maxrank, int level_kind,
                int64_t level);

/* As km_assemble with `d_pts` in device memory of the handle's device (inputs resident in HBM). */
int km_assemble_dev(km_handle* h, const double* d_pts, int64_t n, int kernel_id,
                    const double* params, int nparams, int method, double tol, int64_t maxrank,
                    int level_kind, int64_t level);

/* Rank of every off-diagonal block, level 1 first (nnonleaf entries): size(K.U[l][k], 2) of the
 * reference's KernelHODLR (src/HODLR/src/structstypes.jl:52-63), which has no accessor of its
 * own.  Exposed, with the pivots and factors below, for parity checks. */
int km_block_ranks(km_handle* h, int64_t* out);

/* ACA pivots (0-based within the block) of block `block` (global index, level 1 first):
 * rows and cols receive up to `cap` entries each; *out_rank gets the block rank.  The
 * reference's ACA (src/factorizations.jl:9-84) keeps its pivots internal. */
int km_aca_pivots(km_handle* h, int64_t block, int64_t cap, int64_t* rows, int64_t* cols,
                  int64_t* out_rank);

/* Off-diagonal factors U (rows a:b) and V (rows c:d) of block `block`, column-major with the
 * block rank as column count, as KernelHODLR.U[l][k] / .V[l][k] hold them before
 * factorisation (src/HODLR/src/structstypes.jl:52-63).  Buffers sized (b-a+1)*rank, (d-c+1)*rank. */
int km_block_factors(km_handle* h, int64_t block, double* U, double* V);

/* ---- products, factorisation, solves ------------------------------------------------------ */

/* y = K x for k columns (n x k, column-major).
 * Replaces mul!(target, K::KernelHODLR, src) (src/HODLR/src/baseoverloads.jl:152-179): before
 * factorisation the leaf + U V' form, after it W (W' x). */
int km_matvec(km_handle* h, const double* x, double* y, int64_t k);

/* Symmetric factorisation K = W W'.  Replaces symmetricfactorize!
 * (src/HODLR/src/symfact.jl:6-49). */
int km_factorize(km_handle* h);

/* x = K^{-1} b for k columns.  Replaces ldiv!(target, K::KernelHODLR, src) and \
 * (src/HODLR/src/baseoverloads.jl:181-192, :252-263). */
int km_solve(km_handle* h, const double* b, double* x, int64_t k);

/* x = W^{-1} b (transpose = 0) or W'^{-1} b (transpose = 1).  Replaces ldiv!(t, K.W, v) and
 * ldiv!(t, K.W', v) (src/HODLR/src/baseoverloads.jl:126-150). */
int km_factor_solve(km_handle* h, int transpose, const double* b, double* x, int64_t k);

/* x = W b (transpose = 0) or W' b (transpose = 1).  Replaces mul!(t, K.W, v) and
 * mul!(t, K.W', v) (src/HODLR/src/baseoverloads.jl:95-124). */
int km_factor_mul(km_handle* h, int transpose, const double* b, double* x, int64_t k);

/* log det K.  Replaces logdet(K::KernelHODLR) (src/HODLR/src/baseoverloads.jl:194-209). */
int km_logdet(km_handle* h, double* out);

/* Device-resident variants of km_matvec, km_solve, km_factor_solve and km_factor_mul (the same
 * reference calls): pointers are device memory of the handle's device; the work is ordered on
 * the handle's stream and the call returns once it is complete. */
int km_matvec_dev(km_handle* h, const double* d_x, double* d_y, int64_t k);
int km_solve_dev(km_handle* h, const double* d_b, double* d_x, int64_t k);

/* symmetricfactorize!(HK) then HK \ b in one call (src/HODLR/src/symfact.jl:6-49,
 * src/HODLR/src/baseoverloads.jl:181-192), as LAPACK's posv combines potrf and potrs: the forward
 * half of the solve runs behind the factorisation's dependency points on a second stream.
 * Status, factor and x are those of km_factorize followed by km_solve (_dev: device pointers,
 * in place allowed). */
int km_factorize_solve(km_handle* h, const double* b, double* x, int64_t k);
int km_factorize_solve_dev(km_handle* h, const double* d_b, double* d_x, int64_t k);
int km_factor_solve_dev(km_handle* h, int transpose, const double* d_b, double* d_x, int64_t k);
int km_factor_mul_dev(km_handle* h, int transpose, const double* d_b, double* d_x, int64_t k);

/* Allocation-free solve: x = K^{-1} b for k columns, device pointers, for Nystrom handles.  It
 * has no counterpart in the reference.  It runs the kernels of km_solve_dev in the same order
 * (one conversion to float pairs and back in the mixed form, and the FP64 iterative refinement
 * when the handle's config asks for it), so its result equals km_solve_dev's.  It exists for
 * callers that cannot call cudaMalloc at solve time: cudaMalloc and cudaFree synchronise the
 * whole device (a serving loop that keeps other streams busy cannot afford that), and some hosts
 * hand every byte of device memory to their own pool allocator.  Instead of the handle's growable
 * workspace, the call uses one fixed device array compiled into this library,
 * KM_NOALLOC_SCRATCH_BYTES (8 MiB) large, which every GPU that loads the library holds until the
 * process exits.  The handle must already be factorised (its factor was allocated by
 * km_assemble/km_factorize).  The workspace is 8 * k * r * (2 * (nleaves + nnodes) + 2 * nnodes)
 * bytes, plus 8 * k * (n + 2) for the refinement of a mixed handle and another 8 * n * k when that
 * call runs in place (d_x == d_b); a request above the array, or a refined one of more than 256
 * columns, is rejected with KM_ERR_BAD_ARG: split the columns over several calls.  ACA handles
 * are rejected with KM_ERR_UNSUPPORTED (their solve workspace depends on the block ranks and is
 * grown on demand).  The first call on a device looks up the array's device address with that
 * device current, so make it before any stream capture.  All calls share the array and it keeps
 * the last call's contents (the solve writes every workspace entry before reading it, so nothing
 * needs clearing): calls that overlap on the GPU, from any handle or thread, race on it and must
 * be serialised by the caller. */
#define KM_NOALLOC_SCRATCH_BYTES (8u << 20)
int km_solve_noalloc(km_handle* h, const double* d_b, double* d_x, int64_t k);

/* ---- Gaussian-process likelihood ---------------------------------------------------------- */

/* y' = dK_j x for the exact derivative of the Nystrom HODLR in parameter j (0 scale,
 * 1 range, 2 nugget).  Replaces DerivativeHODLR (src/HODLR/src/constructor.jl:66-95) with
 * mul!(target, DK::DerivativeHODLR, src) (src/HODLR/src/baseoverloads.jl:216-234). */
int km_derivative_matvec(km_handle* h, int param, const double* x, double* y, int64_t k);

/* Negative log-likelihood 0.5 logdet K + 0.5 y'K^{-1}y and its stochastic gradient over the
 * nprobe probe vectors (n x nprobe, column-major) for the 3 kernel parameters.
 * Replaces negloglik (src/HODLR/src/maxlikfunctions.jl:2-9) and stoch_gradient
 * (src/HODLR/src/stochasticgradient.jl:30-44, shuffle = false).  grad may be NULL (NLL only).
 * Requires a factorised Nystrom HODLR. */
int km_nll_grad(km_handle* h, const double* y, const double* probes, int64_t nprobe,
                double* nll, double* grad);

/* km_nll_grad with the probes drawn on the device instead of copied from the host: entry (i, j)
 * of the n x nprobe block is +1 when the top bit of SplitMix64(SplitMix64(seed) + j*n + i) is
 * set, else -1.  Replaces givesaa(n, m; seed) (src/utils.jl:22-27) + stoch_gradient
 * (src/HODLR/src/stochasticgradient.jl:30-44); Julia's own generator is not reproduced, so
 * the probe values differ from the reference's for the same seed (the estimator is the same). */
int km_nll_grad_seeded(km_handle* h, const double* y, int64_t nprobe, uint64_t seed, double* nll,
                       double* grad);

/* Profile likelihood: the scale parameter profiled out.  nll = 0.5 (logdet K + n log(y'K^{-1}y)),
 * grad_j = 0.5 (tr-estimate_j - n y'K^{-1} dK_j K^{-1}y / y'K^{-1}y).  Replaces profile_negloglik
 * (src/HODLR/src/maxlikfunctions.jl:11-19) and stoch_profile_gradient
 * (src/HODLR/src/stochasticgradient.jl:48-86, shuffle = false); the arguments are those of
 * km_nll_grad / km_nll_grad_seeded.  KM_ERR_BAD_ARG when y'K^{-1}y <= 0 (e.g. y = 0), where the
 * reference's log would return -Inf or NaN. */
int km_profile_nll_grad(km_handle* h, const double* y, const double* probes, int64_t nprobe,
                        double* nll, double* grad);
int km_profile_nll_grad_seeded(km_handle* h, const double* y, int64_t nprobe, uint64_t seed,
                               double* nll, double* grad);

/* NLL, stochastic gradient and the stochastic Fisher information matrix from one set of probes:
 * fisher (3 x 3, symmetric, column-major) F_jk = 0.5 mean_v (W^{-1} dK_j W'^{-1} v)'
 * (W^{-1} dK_k W'^{-1} v).  Replaces grad_and_fisher_matrix (src/HODLR/src/stochastichessian.jl:
 * 152-181), fisher_matrix (src/HODLR/src/maxlikfunctions.jl:138-146) and stoch_fisher
 * (stochastichessian.jl:91-115, shuffle = false).  grad and fisher are required, nprobe >= 1. */
int km_grad_fisher(km_handle* h, const double* y, const double* probes, int64_t nprobe,
                   double* nll, double* grad, double* fisher);
int km_grad_fisher_seeded(km_handle* h, const double* y, int64_t nprobe, uint64_t seed,
                          double* nll, double* grad, double* fisher);

/* Stochastic Hessian of the negative log-likelihood with respect to (scale, range, nugget):
 * hess (3 x 3, symmetric, column-major) = -F + for every pair j <= k the trace term
 * 0.5 mean_v t'D2_jk t (t = W'^{-1} v) where the second derivative is not identically zero, and
 * minus half the solve term -u'dK_k K^{-1} dK_j u - u'dK_j K^{-1} dK_k u + u'D2_jk u
 * (u = K^{-1} y); F is the stochastic Fisher matrix of km_grad_fisher from the same probes, and
 * nll and grad are km_grad_fisher's.  D2_jk is the reference's second-derivative product
 * Deriv2mul with its block terms SDBlock_mul / SDBlock_mul_t as written there (they are not the
 * exact second derivative of a Nystrom block).  Replaces stoch_hessian
 * (src/HODLR/src/stochastichessian.jl:117-147, shuffle = false, profile = false) with the
 * second-derivative functions (its d2funs) of the built-in kernels in closed form; pairs with the
 * nugget, and scale-scale for the Matern kernel, are the reference's ZeroFunction case.
 * nprobe >= 1. */
int km_stoch_hessian(km_handle* h, const double* y, const double* probes, int64_t nprobe, double* nll,
                     double* grad, double* hess);
int km_stoch_hessian_seeded(km_handle* h, const double* y, int64_t nprobe, uint64_t seed, double* nll,
                            double* grad, double* hess);

/* Stochastic Hessian of the negative log PROFILE likelihood (the scale profiled out): nll and
 * grad are km_profile_nll_grad's, hess = -F + 0.5 mean_v t'D2_jk t - 0.5 n (s_jk / y'u
 * + (u'dK_j u)(u'dK_k u) / (y'u)^2) with s_jk the solve term of km_stoch_hessian and F its Fisher
 * matrix.  Replaces stoch_hessian(..., profile = true) with HODLR_p_hess_slv
 * (src/HODLR/src/stochastichessian.jl:15-31, 117-147) as called by nlpl_hessian
 * (src/HODLR/src/maxlikfunctions.jl:120-136).  A pair whose second derivative is identically
 * zero (where the reference raises "I didn't implement this speed-up for the profile likelihood")
 * takes the reference's general path with a zero second-derivative function.  nprobe >= 1. */
int km_stoch_profile_hessian(km_handle* h, const double* y, const double* probes, int64_t nprobe,
                             double* nll, double* grad, double* hess);
int km_stoch_profile_hessian_seeded(km_handle* h, const double* y, int64_t nprobe, uint64_t seed,
                                    double* nll, double* grad, double* hess);

/* k-d ordering of n 2-D points (AoS x, y) on the device, the input step of maxlikdata
 * (src/HODLR/src/constructor.jl:171-181), which sorts with NearestNeighbors.KDTree(pts).data.
 * That package's permutation is not reproduced; this library's ordering is: a range of more than
 * `leaf` points is sorted stably by its coordinate of larger spread (max - min, x on a tie), its
 * first floor(len/2) points form the left child, the rest the right child, recursively; ranges of
 * at most `leaf` points keep their order.  perm[i] = original index of sorted position i.
 * Coordinates must be finite; n < 2^31.  Uses the handle's device and stream, not its problem. */
int km_kd_order(km_handle* h, const double* pts, int64_t n, int64_t leaf, int64_t* perm);

/* maxlikdata(pts=, data=, sortmethod=:KDTree) with the ordering of km_kd_order: the sorted points
 * (2 n values) and the data carried with them (data_reorder, src/utils.jl:22-25).  data and
 * data_sorted may be NULL (points only), perm may be NULL.  The reference looks data up by point
 * value, so duplicated points all receive the datum of the last duplicate; here every point keeps
 * its own datum. */
int km_maxlikdata(km_handle* h, const double* pts, const double* data, int64_t n, int64_t leaf,
                  double* pts_sorted, double* data_sorted, int64_t* perm);

/* ---- RKernelHODLR: recursive product-only HODLR of K(x1, x2) ------------------------------- */

/* The recursive HODLR of a not necessarily symmetric or square kernel matrix, replacing
 * RKernelHODLR(K, tol, maxrank, lvl) (src/HODLR/src/constructor.jl:130-161; struct
 * src/HODLR/src/structstypes.jl:22-27).  At every level rows split at floor(n1/2), columns at
 * floor(n2/2); A12 and A21 are compressed by ACA (src/factorizations.jl:9-84), the diagonal
 * blocks after `level` splits are dense.  LogLevel(lv) resolves to FixedLevel(floor(log2(min(n1,
 * n2))) - lv).  x1 (n1 points) and x2 (n2 points) are AoS x, y.  Blocks are numbered A12, A21,
 * then the blocks of A11, then those of A22 (the reference's recursive order).  On failure *out
 * is NULL and km_rhodlr_create_error() gives the message. */
typedef struct km_rhodlr km_rhodlr;
int km_rhodlr_create(const km_config* cfg, const double* x1, int64_t n1, const double* x2, int64_t n2,
                     int kernel_id, const double* params, int nparams, double tol, int64_t maxrank,
                     int level_kind, int64_t level, km_rhodlr** out);
int km_rhodlr_destroy(km_rhodlr* r);
const char* km_rhodlr_create_error(void);
const char* km_rhodlr_last_error(const km_rhodlr* r);
/* Number of ACA blocks, dense leaves and levels; the rank of every ACA block (block order
 * above); the pivots of one block.  The reference's RKernelHODLR keeps these in its fields
 * (structstypes.jl:22-27) without accessors; exposed for parity checks. */
int km_rhodlr_info(const km_rhodlr* r, int64_t* nblocks, int64_t* nleaves, int64_t* levels);
int km_rhodlr_block_ranks(const km_rhodlr* r, int64_t* ranks);
int km_rhodlr_aca_pivots(km_rhodlr* r, int64_t block, int64_t cap, int64_t* rows, int64_t* cols,
                         int64_t* rank);
/* y (n1 x k) = R x (x: n2 x k), host column-major; replaces *(R::RKernelHODLR, V)
 * (src/HODLR/src/baseoverloads.jl:301-305), column by column. */
int km_rhodlr_matvec(km_rhodlr* r, const double* x, double* y, int64_t k);

/* Frees the device buffers of the handle's current problem (the handle stays usable; the next
 * km_assemble allocates again).  No reference counterpart: Julia's GC frees the arrays. */
int km_trim(km_handle* h);

/* Device bytes one handle holds for a Nystrom problem of n points at this rank and level with
 * `ncols` right-hand-side columns (probes + 1 for a likelihood gradient), `with_grad` adding
 * the derivative workspaces.  Pure host arithmetic; -1 for invalid arguments. */
int64_t km_estimate_bytes(int64_t n, int64_t rank, int level_kind, int64_t level, int64_t ncols,
                          int with_grad);

/* ---- batched form: many independent likelihood problems ------------------------------------ */

/* One problem of a batch or serving request.  Host pointers; the caller keeps them valid until
 * the call (batch) or the request (serving) completes. */
typedef struct km_problem {
  int64_t n;             /* number of points                                                  */
  const double* pts;     /* 2*n values, (x, y) pairs, already in the caller's (k-d) order     */
  const double* y;       /* n observations                                                    */
  double params[3];      /* kernel parameters (scale, range, nugget)                          */
} km_problem;

typedef struct km_batch_opts {
  int kernel_id;         /* enum km_kernel_id                                                 */
  int64_t rank;          /* Nystrom rank (the gradient needs Nystrom blocks, constructor.jl:69) */
  int level_kind;        /* enum km_level_kind                                                */
  int64_t level;
  int64_t nprobe;        /* Rademacher probes per problem; 0 => NLL only                      */
  uint64_t probe_seed;   /* problem b draws its probes with seed probe_seed + b               */
  int profile;           /* nonzero => profile likelihood (nlpl_objective,                     */
                         /* src/HODLR/src/maxlikfunctions.jl:61-82) instead of nll_objective  */
} km_batch_opts;

typedef struct km_batch km_batch;

/* A pool of `nworkers` handles (0 => 8), each with its own stream and host thread, that keeps
 * its device buffers between calls (grown to the largest problem seen).  No reference
 * counterpart (see km_batch_nll_grad). */
int km_batch_create(const km_config* cfg, int nworkers, km_batch** out);
int km_batch_destroy(km_batch* b);

/* For every problem b: assemble (Nystrom), symmetricfactorize!, negloglik and, when nprobe > 0,
 * the stochastic gradient.  nll[b], grad[3*b .. 3*b+2] and status[b] (enum km_status) are
 * written per problem; one failing problem does not stop the others.  Problems are dispatched
 * largest first to the workers, which run concurrently on the GPU.  Replaces the loop a caller
 * writes around nll_objective (src/HODLR/src/maxlikfunctions.jl:29-50) for independent
 * datasets; the reference has no batched entry point.  Returns KM_OK when every problem
 * succeeded, else the first failing status (message in km_batch_last_error). */
int km_batch_nll_grad(km_batch* b, const km_batch_opts* o, int64_t nprob, const km_problem* probs,
                      double* nll, double* grad, int* status);
const char* km_batch_last_error(const km_batch* b);

/* ---- serving form: continuous batching with HBM-budget admission --------------------------- */

enum km_req_kind {
  KM_REQ_NLL_GRAD = 0,   /* negloglik (+ stochastic gradient when nprobe > 0) of `prob`        */
  KM_REQ_FACTOR = 1,     /* assemble + factorise `prob` and keep the factor resident          */
  KM_REQ_SOLVE = 2,      /* x = K^{-1} b with the resident factor `factor_id` (nrhs columns)  */
  KM_REQ_RELEASE = 3,    /* drop the resident factor `factor_id`                               */
  KM_REQ_PROFILE_NLL_GRAD = 4 /* profile_negloglik (+ stoch_profile_gradient) of `prob`       */
};

typedef struct km_request {
  int kind;              /* enum km_req_kind                                                  */
  km_problem prob;       /* NLL_GRAD, PROFILE_NLL_GRAD, FACTOR                                */
  int64_t nprobe;        /* NLL_GRAD, PROFILE_NLL_GRAD                                        */
  uint64_t probe_seed;   /* NLL_GRAD, PROFILE_NLL_GRAD                                        */
  int64_t factor_id;     /* SOLVE, RELEASE                                                    */
  const double* b;       /* SOLVE: n x nrhs right-hand sides (host, column-major)              */
  double* x;             /* SOLVE: n x nrhs solutions (host, column-major)                     */
  int64_t nrhs;          /* SOLVE                                                             */
} km_request;

typedef struct km_result {
  int status;            /* enum km_status of the request                                     */
  double nll;            /* NLL_GRAD                                                          */
  double grad[3];        /* NLL_GRAD with nprobe > 0                                          */
  double logdet;         /* FACTOR                                                            */
  int64_t factor_id;     /* FACTOR: id for later SOLVE / RELEASE requests                     */
  double queue_ms;       /* submit -> start                                                   */
  double run_ms;         /* start -> end                                                      */
} km_result;

typedef struct km_serve_opts {
  int kernel_id;
  int64_t rank;
  int level_kind;
  int64_t level;
  int nworkers;          /* concurrent executors (0 => 8)                                     */
} km_serve_opts;

typedef struct km_serve_stats {
  int64_t submitted, completed, failed, rejected;
  int64_t resident_factors;
  int64_t bytes_in_use;  /* device bytes held by executors and resident factors               */
  int64_t peak_bytes;
  int64_t budget_bytes;  /* hbm_budget_fraction of the device's memory                        */
  double p50_ms, p99_ms, mean_ms;  /* submit -> completion latency of completed requests      */
} km_serve_stats;

typedef struct km_server km_server;

/* Starts the scheduler thread and `nworkers` executors.  A request is admitted when its
 * estimated device bytes fit in the budget next to everything in flight and resident;
 * admission is first-come first-served with later requests allowed to pass one that does
 * not fit yet.  A request that cannot fit even on an idle server fails with KM_ERR_OOM.
 * No reference counterpart (the reference is a library called in-process). */
int km_serve_create(const km_config* cfg, const km_serve_opts* o, km_server** out);

/* Queues a request; *ticket identifies it for km_serve_wait.  This and the calls below have no
 * reference counterpart, like km_serve_create. */
int km_serve_submit(km_server* s, const km_request* r, uint64_t* ticket);

/* Waits up to timeout_ms (< 0: forever) for the request; KM_ERR_TIMEOUT if still running.
 * A result is returned once; its ticket is then forgotten. */
int km_serve_wait(km_server* s, uint64_t ticket, int64_t timeout_ms, km_result* out);

int km_serve_stats_get(km_server* s, km_serve_stats* out);

/* Drains every queued and running request, releases resident factors and stops the threads. */
int km_serve_destroy(km_server* s);

/* ---- streams and profiling ---------------------------------------------------------------- */

/* Runs the handle's work on `stream` (a cudaStream_t of the handle's device; NULL restores the
 * handle's own stream).  The caller keeps ownership of the stream.  The streams, profiling and
 * diagnostics calls below have no reference counterpart (the reference runs on the host). */
int km_set_stream(km_handle* h, void* stream);

/* Kernel classes timed by the profiler. */
enum km_prof_class {
  KM_PROF_EVAL = 0,        /* kernel-entry evaluation (leaves, landmark columns, S)           */
  KM_PROF_LEAF_CHOL = 1,   /* batched leaf Cholesky                                           */
  KM_PROF_LEAF_TRI = 2,    /* leaf triangular solves / products                               */
  KM_PROF_LEAF_QR = 3,     /* leaf Householder QR                                             */
  KM_PROF_NODE = 4,        /* per-level node factorisation                                    */
  KM_PROF_SWEEP = 5,       /* up/down tree sweeps of products and solves                      */
  KM_PROF_LEAF_REFL = 6,   /* leaf reflector projections / expansions                         */
  KM_PROF_LEAF_APPLY = 7,  /* leaf products of the HODLR matvec                               */
  KM_PROF_OTHER = 8,       /* small kernels (logdet reduction, landmark Cholesky, ...)        */
  KM_PROF_ACA = 9,         /* adaptive cross approximation                                    */
  KM_PROF_LEAF_TC = 10,    /* tensor-core trailing updates of the mixed-form leaf Cholesky     */
  KM_PROF_COUNT = 11
};

/* Enables (1) or disables (0) per-launch CUDA-event timing; enabling clears the counters. */
int km_profile_enable(km_handle* h, int on);

/* Accumulated device time (ms) and launch count of kernel class `cls` since enabling. */
int km_profile_get(km_handle* h, int cls, double* total_ms, int64_t* launches);

/* ---- diagnostics ------------------------------------------------------------------------- */

/* Number of polls after which a bounded device-side wait of this handle's kernels gives up: the
 * dataflow flags of the mixed-form node factorisation and the grid barriers of the ACA and tall
 * panel-QR kernels.  polls < 0 restores the defaults (well above any legitimate wait); 0 makes
 * every such wait give up at its first poll, as if the flag it waits for were never set.  A wait
 * that gives up ends its kernel early and the call returns KM_ERR_TIMEOUT; the handle stays
 * usable (assemble again).  For tests of that path.  No reference counterpart. */
int km_set_wait_limit(km_handle* h, int64_t polls);

/* Device FP64 FMA throughput in TFLOP/s measured by a short timed loop (roofline denominator
 * for FP64-ALU-bound kernels). */
int km_probe_fp64_tflops(int device, double* out);

/* Device FP32 FMA throughput in TFLOP/s (denominator for the float-pair kernels of the mixed
 * form, which run on the FP32 pipe). */
int km_probe_fp32_tflops(int device, double* out);

/* The tensor-core split product of the mixed-form leaf stage on one tile (host pointers):
 * C = A B' for A (128 x 64) and B (64 x 64), row-major doubles, C 128 x 64 row-major.  mode 0:
 * A and B hold integers of magnitude <= 128, passed to the tensor cores as single bf16 slices,
 * and C is their fp32 sum (exact); mode 1: A and B are rounded to float pairs, cut into slices
 * and multiplied as in the leaf updates.  Used to check the tensor-core data layout and the
 * accuracy of the split product.  No reference counterpart. */
int km_probe_tc_gemm(int device, const double* A, const double* B, int mode, double* C);

#ifdef __cplusplus
}
#endif
#endif /* KMHODLR_H */
