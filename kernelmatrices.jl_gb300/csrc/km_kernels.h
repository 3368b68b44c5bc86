// Launch wrappers of the device kernels (defined in km_assemble.cu, km_factor.cu, km_apply.cu,
// km_aca.cu, km_grad.cu).  Host orchestration lives in km_api.cu.
#pragma once
#include "km_internal.h"
#include "km_ff.cuh"

namespace km {

// Raises the dynamic shared-memory limit of kernel `func` on the current device so that a launch
// may request `bytes`.  The limit is set once per kernel and device to the device's opt-in
// maximum and never lowered, so host threads that launch the same kernel with different sizes
// (the batched and serving forms) cannot shrink it under one another's launches.
void smem_limit(const void* func, size_t bytes);


// Operand of the leaf triangular kernels: leaf j's block starts at ptr + start(j) * bmul with
// leading dimension m_j (ld_is_m) or ld.
struct LeafOperand {
  double* ptr;
  int64_t bmul;
  int64_t ld;
  int ld_is_m;
};

// ---- general (ACA) path descriptors ----
struct AcaBlock {             // rows = second child (a:b), cols = first child (c:d), 0-based
  int64_t row0, nro, col0, ncl;
  int64_t offU, offV;         // column-major U (nro x cap), V (ncl x cap) in the panel arena
  int64_t offFlag, offPiv;    // used-row/col flags (nro + ncl bytes); pivots (2 * cap ints at 2*offPiv)
  int cap, maxsz;
  int grid;                   // 1: large block, compressed by the grid-wide ACA kernel
};
struct PanelDesc {            // Householder QR with explicit Q of A (m x k, leading dim lda)
  double* A;
  int64_t m, lda;
  int k;
  double* R;                  // k x k output
  int big;                    // 1: block reflectors applied with library GEMMs (k_pq_update skips it)
};
struct GNodeDesc {            // one node of the general factorisation
  double* Q1;                 // V panel (rows c1), Q after the QR
  double* Q2;                 // U panel (rows c2)
  double* C;
  double* L22;
  const double* R1;
  const double* R2;
  int64_t s1, s2;
  int r;
};
struct GApplyItem {           // node factor applied to rows off1.. (c1) and off2.. (c2) of a block
  int node;
  int ncols;
  int64_t off1, off2, ld;
  double* base;               // nullptr: the right-hand-side block passed to the kernel
  int big;                    // 1: applied with library GEMMs by the host path (k_gapply skips it)
};
struct LeafDesc {             // leaf triangular operation on an arbitrary column block
  int64_t leaf;
  double* ptr;                // first row of the leaf's rows in the block
  int64_t ld;
  int ncols;
};

struct NodeMatsH {          // node factors (double or float pairs, by the caller's precision)
  const void* Ct;
  const void* L22;
  const void* L22i;
  const void* E;           // explicit 2r x r transfer
  int r;
  // transposed copies (r x r, r x 2r for E^T), so that every sweep product reads coalesced rows
  const void* CtT = nullptr;
  const void* L22T = nullptr;
  const void* L22iT = nullptr;
  const void* ET = nullptr;
};

// assembly
// use_ff: float-pair evaluation on the FP32 pipe (mixed form, ~1e-14 relative), else FP64
// Kff: also the float-pair entries of the kernel itself (mixed form, deriv < 0), lower triangle
void launch_eval_leaves(const double* pts, const Tree& t, KParams kp, int deriv, double* K,
                        cudaStream_t st, bool use_ff = false, ff* Kff = nullptr, const float* P3 = nullptr);
void launch_eval_phi(const double* pts, const double* lnd, int r, const Tree& t, KParams kp,
                     int deriv, double* Phi, cudaStream_t st, bool use_ff = false, const float* P3 = nullptr,
                     const float* L3 = nullptr, ff* Phif = nullptr);
// P3: 8 floats a point, the exact float triples of x and y (km_kfun.cuh), for the float-pair
// evaluations
void launch_split_points(const double* pts, int64_t n, float* P3, cudaStream_t st);
void launch_eval_dense(const double* a, int na, const double* b, int nb, KParams kp, int deriv,
                       double* out, int ld, cudaStream_t st);
void launch_gather_points(const double* pts, const int64_t* idx, int r, double* lnd,
                          cudaStream_t st);

// factorisation
bool launch_chol_small(double* A, int n, int* info, cudaStream_t st);
template <typename T>
bool launch_leaf_chol(const double* K, T* Lf, const Tree& t, int* info, cudaStream_t st);
template <typename T>
bool launch_leaf_tri(const T* Lf, const Tree& t, int op, T* Bptr, int64_t bmul, int64_t bld, int bld_is_m, T* Xptr,
                     int64_t xmul, int64_t xld, int xld_is_m, int ncols, cudaStream_t st);
template <typename T>
void launch_leaf_qr(T* Pan, int r, const Tree& t, T* tau, T* Rout, cudaStream_t st);
// Mixed form on the tensor cores (km_leaf_tc.cu): blocked Cholesky of the augmented leaf matrices
// [K_j; Phi_j'] giving Lf_j (float pairs) and A_j = L_j^{-1} Phi_j in place of G (= the float-pair
// Phi, m x r per leaf).  Lf holds the float-pair leaf matrices (lower triangles) on entry.  Step
// p: the diagonal-block launch, the block-column launch, then (when has_update) the trailing
// update.  scratch: leaf_chol_tc_scratch_bytes(t, r) bytes; info as launch_leaf_chol (-1: a
// bounded wait of a tensor-core launch ran out).
bool leaf_chol_tc_supported(const Tree& t, int r);
// L x = b (op 0) or L' x = b (op 1) on every leaf with a factor of the tensor-core stage (it
// keeps the inverses of its 64 x 64 diagonal blocks), k columns of X in place (ld ldx); false if
// the shape is not supported
bool launch_leaf_tri_blk(const ff* Lf, const Tree& t, int op, ff* X, int64_t ldx, int k, cudaStream_t st);
int64_t leaf_chol_tc_scratch_bytes(const Tree& t, int r);
int leaf_chol_tc_steps(const Tree& t);
bool leaf_chol_tc_has_update(const Tree& t, int p);
void launch_leaf_chol_tc_diag(ff* Lf, int r, const Tree& t, int p, void* scratch, int* info, cudaStream_t st);
void launch_leaf_chol_tc_trsm(ff* Lf, ff* G, int r, const Tree& t, int p, void* scratch, int* info,
                              cudaStream_t st);
void launch_leaf_chol_tc_update(ff* Lf, ff* G, int r, const Tree& t, int p, void* scratch, int* info,
                                cudaStream_t st);
void launch_tri_inv_t(const double* Sc, int r, double* SinvT, cudaStream_t st);
template <typename T>
// wait_limit: polls of a dataflow flag before a wait gives up (< 0: the kernel's default, 0: at
// the first poll, the test of the timeout path); a wait that gives up sets info = -1
void launch_node_factor(T* R, const T* SinvT, int r, int level, const Tree& t, T* Ct, T* L22, T* Eref, T* Etau,
                        int* info, cudaStream_t st, int max_cluster = 8, int wait_limit = -1);
template <typename T>
void launch_leaf_formq(T* Pan, const T* tau, int r, const Tree& t, cudaStream_t st);
template <typename T>
void launch_node_finalize(const T* L22, const T* Ct, const T* Eref, const T* Etau, int r, int level, const Tree& t,
                          T* L22i, T* Eexp, T* CtT, T* L22T, T* L22iT, T* ET, cudaStream_t st);
template <typename T>
void launch_logdet(const T* Lf, const Tree& t, const T* L22, int r, double* partial, int np, double* out,
                   cudaStream_t st);
void launch_to_ff(const double* in, ff* out, int64_t n, cudaStream_t st);
// out[0] = sum of partial[0 .. np) in index order (one thread)
void launch_sum_partials(const double* partial, int np, double* out, cudaStream_t st);
void launch_from_ff(const ff* in, double* out, int64_t n, cudaStream_t st);

// products and solves
enum { UP_PROJ_ = 0, UP_FWD_ = 1, UP_MULT_ = 2, UP_SUM_ = 3 };
// Nystrom sibling sums without the tree: VG = (sum over the leaves of VP) - VP per leaf slot
// (W values a column, k columns)
void launch_nys_sums(const double* VP, double* VG, int64_t nleaf, int W, int k, cudaStream_t st);
template <typename T>
void launch_slot_sub(T* VP, const T* VG, int64_t count, cudaStream_t st);
enum { DN_FWD_ = 0, DN_BWD_ = 1, DN_MUL_ = 2, DN_MULT_ = 3 };
template <typename T>
void launch_up(const Tree& t, const NodeMatsH& h, int level, T* VP, T* VD, int k, int mode, cudaStream_t st);
template <typename T>
void launch_down(const Tree& t, const NodeMatsH& h, int level, const T* VP, T* VG, const T* VD, int k, int mode,
                 cudaStream_t st);
template <typename T>
void launch_leaf_proj(const T* Qref, const T* tau, int r, const Tree& t, const T* Y, int64_t ldy, T* VP, int k,
                      cudaStream_t st);
template <typename T>
void launch_leaf_expand(const T* Qref, const T* tau, int r, const Tree& t, const T* VG, T* Y, int64_t ldy, int k,
                        double sign, cudaStream_t st);
void launch_leaf_phiT(const double* Phi, int r, const Tree& t, const double* X, int64_t ldx,
                      double* VP, int k, cudaStream_t st);
void launch_leaf_nys_apply(const double* Kl, const double* Phi, const double* Sc, int r,
                           const Tree& t, const double* X, int64_t ldx, const double* VG,
                           double* Y, int64_t ldy, int k, cudaStream_t st);

// derivative HODLR and gradient pieces
template <typename T>
void launch_leaf_dphiT(const T* Phi, const T* dPhi, int r, const Tree& t, const double* X, int64_t ldx, double* VP,
                       int k, cudaStream_t st);
template <typename T>
void launch_leaf_dnys_apply(const T* dKl, const T* Phi, const T* dPhi, const double* Sc, const double* Sj, int r,
                            const Tree& t, const double* X, int64_t ldx, const double* VG, double* Y, int64_t ldy,
                            int k, cudaStream_t st, const T* betas = nullptr);
// C = A op(B), r x r FP64 (op = transpose when transB)
// second-derivative product of the stochastic Hessian (km_grad.cu)
void launch_leaf_phi4T(const double* Phi, const double* Phi3, int r, const Tree& t, const double* X, int64_t ldx,
                       double* VP, int k, cudaStream_t st);
void launch_d2_down(const double* Tmul, const double* Tmult, int r, const Tree& t, int level, const double* VP,
                    double* VG, int k, cudaStream_t st);
void launch_leaf_d2_apply(const double* D2, const double* Phi, const double* Phi3, int r, const Tree& t,
                          const double* X, int64_t ldx, const double* VG, double* Y, int64_t ldy, int k,
                          cudaStream_t st);
void launch_d2_assemble(const double* M, int r, double* Tmul, double* Tmult, cudaStream_t st);
void launch_small_gemm(const double* A, const double* B, int r, int transB, double* C, cudaStream_t st);
// landmark coefficients of the derivative products from explicit S^{-1} and S^{-1} Sj S^{-1}
template <typename T>
void launch_dbeta(const T* Sinv, const T* M2, int r, const double* VG, int64_t npairs, T* beta, cudaStream_t st);
void launch_axpby(double* y, const double* x, double a, double b, int64_t n, cudaStream_t st);
// trace form of the stochastic gradient (km_grad.cu).  X: n x k (k = p + 1: p probes with weight
// 1/p, then alpha with weight wa); W = 4r projection rows per (leaf, column) pair.
template <typename T>
void launch_eval_dphi2(const double* pts, const double* lnd, const float* P3, const float* L3, int r, const Tree& t,
                       KParams kp, T* dPhi2, cudaStream_t st);
template <typename T>
void launch_leaf_proj3(const T* Phi, const T* dPhi2, int r, const Tree& t, const T* X, int64_t ldx, double* VP, int k,
                       cudaStream_t st);
void launch_nugget_proj(const double* pts, const double* lnd, int r, const Tree& t, const double* X, int64_t ldx,
                        double* VP, int k, cudaStream_t st);
void launch_proj_total(double* VP, int W, int64_t nleaf, int k, cudaStream_t st);
template <typename T>
void launch_landmark(const double* VP, int r, int k, int p, double wa, const T* Sinv, const T* Sj3, int64_t nleaf,
                     double* part, cudaStream_t st);
int leaf_dk_gram_parts(const Tree& t);  // CTAs per leaf of the leaf term (partial sums per leaf)
template <typename T>
void launch_leaf_dk_gram(const double* pts, const float* P3, KParams kp, const T* X, int64_t n, int p, double wa,
                         const Tree& t, double* part, cudaStream_t st);
// out[j] = scale * (sum_q a[j * na + q] + sum_q b[j * nb + q]) for j < 3, fixed order
void launch_grad_final(const double* a, int64_t na, const double* b, int64_t nb, double scale, double* out,
                       cudaStream_t st);
// n x p Rademacher probes (+-1), entry (i, j) from a SplitMix64 hash of (seed, j*n + i)
void launch_rademacher(double* out, int64_t n, int64_t p, uint64_t seed, cudaStream_t st);
void launch_col_dots(const double* A, int64_t lda, const double* B, int64_t ldb, int64_t n, int k,
                     double* out, cudaStream_t st);

// ACA and the general factorisation
constexpr int kAcaMaxCap = 4096;       // ACA panel columns per block (2 x 4096 doubles of shared memory)
constexpr int64_t kAcaGridMin = 8192;  // blocks at least this wide run the grid-wide ACA kernel
void launch_aca(const double* pts, KParams kp, const AcaBlock* blocks, int nblocks, int maxcap, double* P,
                uint8_t* F, int* piv, double rtol, int* rank, int* status, cudaStream_t st);
// ACA of one large block (blocks[b].grid == 1) by all SMs in one cooperative launch, with
// bounded grid barriers; scratch of aca_grid_scratch(cap) doubles.  Returns false when the
// cooperative launch is unavailable (the caller then runs the block in the one-CTA kernel).
// wait_limit: polls before a grid barrier gives up (< 0: default; 0: at the first poll)
bool launch_aca_grid(const double* pts, KParams kp, const AcaBlock* blocks, int b, int cap, double* P, uint8_t* F,
                     int* piv, double rtol, int* rank, int* status, double* scratch, cudaStream_t st,
                     long long wait_limit = -1);
int64_t aca_grid_scratch(int cap);
// one-CTA ACA of a single block regardless of its grid flag (fallback)
void launch_aca_one(const double* pts, KParams kp, const AcaBlock* blocks, int b, int maxcap, double* P,
                    uint8_t* F, int* piv, double rtol, int* rank, int* status, cudaStream_t st);
// Householder QR with explicit Q of n panels (largest column count kmax); scratch of
// panel_qr_scratch(n, kmax) doubles: taus (n x kmax) then the T factors
void launch_panel_qr(const PanelDesc* descs, int n, int kmax, double* taus, double* Ts, cudaStream_t st);
// the same with the panels marked big handled by all SMs: their 8-column factor and form steps
// as cooperative launches (bounded grid barriers; a barrier that runs out sets *grid_err) and
// their block-reflector applications as FP64 products over all SMs (launch_dgemm; hdescs: host
// copies of descs;
// gemm_scratch: panel_qr_gemm_scratch(hdescs, n, kmax) doubles)
void launch_panel_qr_gemm(const PanelDesc* descs, const PanelDesc* hdescs, int n, int kmax, double* taus,
                          double* Ts, double* gemm_scratch, int* grid_err, cudaStream_t st,
                          long long wait_limit = -1);
int64_t panel_qr_gemm_scratch(const PanelDesc* hdescs, int n, int kmax);
// C = alpha op(A) B + beta C (FP64, column-major; op(A) = A' when transA), km_gemm.cu.  A long
// reduction with op = T is split over CTAs when `scratch` holds dgemm_scratch(...) doubles
// (scratch_len of them; fewer splits if it holds less, none if null).
void launch_dgemm(int transA, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                  const double* B, int64_t ldb, double beta, double* C, int64_t ldc, double* scratch,
                  int64_t scratch_len, cudaStream_t st);
int64_t dgemm_scratch(int transA, int64_t M, int64_t N, int64_t K);
int64_t panel_qr_scratch(int n, int kmax);
void launch_gnode(const GNodeDesc* nodes, int n, int* info, cudaStream_t st);
void launch_gapply(const GApplyItem* items, int n, const GNodeDesc* nodes, int maxr, int maxcols, int mode,
                   double* X, const double* Xin, int64_t ldX, int kX, cudaStream_t st);
void launch_glogdet(const GNodeDesc* nodes, int nn, double* partial, cudaStream_t st);
// the r x r part of k_gapply for one node and ncols columns: from the projections Z1 = Q1' x1,
// Z2 = Q2' x2 (r x ncols each; mode 4 is not handled here) to the expansion coefficients G1, G2
void launch_gsmall(const GNodeDesc* node, int mode, const double* Z1, const double* Z2, double* G1, double* G2,
                   int r, int ncols, cudaStream_t st);
bool launch_leaf_tri_desc(const double* Lf, const Tree& t, int op, const LeafDesc* descs, int n, int maxcols,
                          cudaStream_t st);

// k-d ordering of 2-D points (km_kd.cu): a contiguous range of positions, split or final
struct KdSeg {
  int64_t start, len;
  int split;
};
size_t kd_scratch_bytes(int64_t n);
bool kd_order_device(const double* d_pts, int64_t n, int64_t leaf, int64_t* d_perm, void* d_scratch,
                     cudaStream_t st, std::string* err);
// pts_s[i] = pts[perm[i]] (2-D), data_s[i] = data[perm[i]] when data is not null
void launch_gather_sorted(const double* pts, const double* data, const int64_t* perm, int64_t n, double* pts_s,
                          double* data_s, cudaStream_t st);

}  // namespace km
