// C ABI of libkmhodlr: handle lifecycle, partition, and the orchestration of the device kernels.
// Each entry point mirrors one reference call (cited in include/kmhodlr.h).
#include <algorithm>
#include <type_traits>
#include <mutex>
#include <cmath>
#include <cstdlib>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "km_kernels.h"

using namespace km;

// ---------------------------------------------------------------------------------------------
// tree partition (src/HODLR/src/indices.jl)
// ---------------------------------------------------------------------------------------------
namespace km {

bool build_tree(int64_t n, int level_kind, int64_t level, Tree* t, std::string* msg) {
  if (n < 1 || n >= (int64_t(1) << 48)) {
    *msg = "n must satisfy 1 <= n < 2^48";
    return false;
  }
  if (level_kind != KM_LEVEL_FIXED && level_kind != KM_LEVEL_LOG) {
    *msg = "level_kind must be KM_LEVEL_FIXED or KM_LEVEL_LOG";
    return false;
  }
  // floor(log2(n)) is exact for n < 2^48 (indices.jl:7,10)
  int fl = 0;
  while ((n >> (fl + 1)) > 0) ++fl;
  int64_t L;
  if (level_kind == KM_LEVEL_FIXED) {
    L = std::min<int64_t>(std::max<int64_t>(0, level), fl);
  } else {
    if (level < 0) {
      *msg = "Please provide a positive value for the level offset.";
      return false;
    }
    L = std::min<int64_t>(std::max<int64_t>(0, fl - level), fl);
  }
  if (L > kMaxLevels) {
    *msg = "too many levels";
    return false;
  }
  t->n = n;
  t->L = (int)L;
  t->nleaf = int64_t(1) << L;
  t->m0 = n >> L;                       // floor(n / 2^L)
  t->rem = n - t->m0 * t->nleaf;        // the first `rem` leaves get one more point
  t->nnode = t->nleaf - 1;
  t->max_leaf = t->m0 + (t->rem > 0 ? 1 : 0);
  t->node_off.assign(t->L + 2, 0);
  for (int l = 1; l <= t->L; ++l) t->node_off[l + 1] = t->node_off[l] + t->nodes_at(l);
  return true;
}

}  // namespace km

// ---------------------------------------------------------------------------------------------
// handle
// ---------------------------------------------------------------------------------------------
struct km_handle {
  km_config cfg{};
  cudaStream_t stream = nullptr;
  std::string err;
  km_stats stats{};
  std::vector<std::pair<void*, size_t>> allocs;  // problem-lifetime device buffers
  int64_t bytes = 0;

  bool assembled = false, factorized = false;
  Tree tree;
  KParams kp{};
  int method = KM_METHOD_NYSTROM;
  bool mixed = false;  // float-pair factor (KM_PREC_MIXED)
  bool leaf_tc = false;  // mixed form: leaf Cholesky and L^{-1} Phi on the tensor cores
  bool lf_holds_k = false;  // d_Lf holds the float-pair leaf matrices (written by the assembly)
  bool q_holds_phi = false;  // d_Q holds Phi as float pairs (written by the mixed assembly)
  double* d_lcscr = nullptr;  // slices and row exponents of the tensor-core leaf stage
  // CTAs per node of the float-pair node kernel at most (thread-block clusters on levels with
  // few nodes); 1 for handles of the batch and serving pools, whose streams fill the SMs already
  int node_cluster_max = 8;
  int64_t wait_limit = -1;  // polls before a bounded device wait gives up (km_set_wait_limit)
  double tol = 0.0;
  int64_t maxrank = 0;
  int r = 0;

  double* d_pts = nullptr;
  double* d_lnd = nullptr;
  float* d_pts3 = nullptr;  // mixed form: points and landmarks as exact float triples (km_kfun.cuh)
  float* d_lnd3 = nullptr;
  int64_t* d_lndidx = nullptr;
  double* d_K = nullptr;
  double* d_Lf = nullptr;
  double* d_Phi = nullptr;
  double* d_Q = nullptr;
  double* d_tauleaf = nullptr;
  double* d_R = nullptr;
  double* d_S = nullptr;
  double* d_Sc = nullptr;
  double* d_SinvT = nullptr;
  double* d_SinvTf = nullptr;  // float-pair copy for the mixed form
  double* d_Ct = nullptr;
  double* d_L22 = nullptr;
  double* d_Eref = nullptr;
  double* d_Etau = nullptr;
  double* d_L22i = nullptr;  // L22^{-1} per node
  double* d_E = nullptr;     // explicit 2r x r transfer per node
  double* d_NT = nullptr;    // transposes per node: Ct', L22', L22^{-1}', E' (5 r^2 per node)
  int* d_info = nullptr;
  double* d_partial = nullptr;
  double* d_scalar = nullptr;
  // workspaces that grow with the column count
  double* d_VP = nullptr;
  double* d_VG = nullptr;
  double* d_VD = nullptr;
  int64_t vcap = 0;
  double* d_X = nullptr;
  double* d_Y = nullptr;
  int64_t xcap = 0;
  // general (ACA) path
  std::vector<AcaBlock> blk;          // off-diagonal blocks, level 1 first
  std::vector<int> brank;             // ACA rank per block
  std::vector<int64_t> lvoff;         // first block of each level (size L+2, lvoff[l] for l=1..L+1)
  AcaBlock* d_blk = nullptr;
  double* d_panels = nullptr;
  uint8_t* d_flags = nullptr;
  int* d_piv = nullptr;
  int* d_brank = nullptr;
  int* d_bstatus = nullptr;
  double* d_R12 = nullptr;
  double* d_CL = nullptr;
  GNodeDesc* d_gnodes = nullptr;
  GApplyItem* d_gsolve = nullptr;     // one item per block, rows relative to the right-hand side
  GApplyItem* d_gfact = nullptr;      // factorisation updates, grouped by level
  std::vector<GNodeDesc> gnodes_h;    // host copies: the library-GEMM path of large nodes reads them
  std::vector<GApplyItem> gsolve_h, gfact_h;
  double* d_gz = nullptr;             // projections and coefficients of one large node (4 x r x ncols),
                                      // then the partial products of its split projections
  double* d_pqg = nullptr;            // explicit reflector block and products of the tall-panel QR
  std::vector<int64_t> gfoff;
  PanelDesc* d_pdesc = nullptr;
  LeafDesc* d_ldesc = nullptr;
  int64_t nldesc = 0;
  int gmaxr = 0;
  double* d_gpartial = nullptr;
  double* d_pqs = nullptr;            // panel QR scratch (taus, block reflector T factors)
  double* d_acascr = nullptr;         // grid-wide ACA scratch (per-CTA records, barrier words)
  // derivative HODLR (evaluated for one parameter at a time) and gradient workspaces
  int dk_param = -1;
  double* d_dK = nullptr;
  double* d_dPhi = nullptr;
  double* d_Sj = nullptr;
  double* d_Sinv = nullptr;   // mixed form: explicit S^{-1} and S^{-1} Sj S^{-1} (FP64 + float pairs)
  double* d_SinvF = nullptr;
  double* d_M2 = nullptr;
  double* d_M2F = nullptr;
  double* d_Mtmp = nullptr;
  double* d_GB = nullptr;     // mixed form: landmark coefficients of the leaf derivative products
  double* d_dKf = nullptr;    // float-pair copies (mixed form) of dK leaves, dPhi and Phi
  double* d_dPhif = nullptr;
  double* d_Phif = nullptr;
  double* d_GP = nullptr;
  double* d_GG = nullptr;
  int64_t gcap = 0;
  double* d_T = nullptr;
  double* d_U = nullptr;
  double* d_dots = nullptr;
  int64_t tcap = 0;
  double* d_A = nullptr;     // Fisher: W^{-1} dK_j W'^{-1} V for the three parameters (3 n x p)
  // stochastic Hessian: second-derivative product, evaluated for one parameter pair at a time
  int d2_pair = -1;           // evaluation code (kD2Base + 3 j + k) of the cached pair, -1 none
  double* d_hPhi3 = nullptr;  // Phi_j, Phi_k, Phi_jk (3 n r, the per-leaf layout of Phi)
  double* d_hD2 = nullptr;    // dense second-derivative leaves
  double* d_hS = nullptr;     // Sj, Sk, Sjk, three products with S^{-1}, then A, Bj, Bk, Bjk, Cjk, Ckj
  double* d_hT = nullptr;     // Tmul, Tmult ((4r)^2 each)
  double* d_hP = nullptr;     // per slot and column: four projections (4r) ...
  double* d_hG = nullptr;     // ... and four expansion coefficients (4r)
  int64_t hcap = 0;
  double* d_hA = nullptr;     // a_j = dK_j u and b_j = K^{-1} a_j (6 n)
  double* d_hY = nullptr;     // second-derivative products of [W'^{-1} V | u]
  double* d_hdots = nullptr;
  double* d_dPhi2 = nullptr;  // trace-form gradient: dK_j(X, P) for j = 0, 1 (float pairs when mixed)
  double* d_Sj3 = nullptr;    // dK_j(P, P), j = 0, 1, 2
  double* d_Sj3F = nullptr;   // float-pair copy (mixed form)
  double* d_VP4 = nullptr;    // projections [phi ; dphi_0 ; dphi_1 ; dphi_2] per (leaf, column), then the sums
  double* d_gpart = nullptr;  // per-leaf partial sums of the trace-form gradient, then 3 sums
  double* d_res = nullptr;   // refinement residual (n x rcap)
  double* d_rdots = nullptr;
  int64_t rcap = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaStream_t own_stream = nullptr;  // the handle's own stream (h->stream may be external)
  cudaStream_t side = nullptr;        // forms the solve operators while the node levels run
  cudaEvent_t sev[kMaxLevels + 3] = {};
  // fused factorisation and solve (km_factorize_solve_dev): the forward half of the solve runs on
  // `aux` behind the factorisation's dependency points (leaf factor ready: xev[0]; explicit leaf
  // bases: xev[1]; node level l finalised: fev[l]; forward half done: xev[2])
  cudaStream_t aux = nullptr;
  cudaEvent_t xev[3] = {};
  double* d_bkeep = nullptr;  // right-hand sides kept by an in-place fused call
  // pinned host copy of the pivot status words (d_info), filled by an asynchronous copy that the
  // call's closing synchronisation covers: no separate round trip to read them
  int* h_info = nullptr;
  int64_t h_info_cap = 0;
  cudaEvent_t fev[kMaxLevels + 2] = {};
  struct FwdJob {
    double* X;
    int k;
    bool ok;
  }* fwd_job = nullptr;
  // profiler
  bool prof = false;
  // CUDA graphs of the launch sequences of a Nystrom factorisation and of a nested solve,
  // replayed while the handle's buffers (alloc_epoch) and the shapes in the key are unchanged
  uint64_t alloc_epoch = 0;
  cudaGraphExec_t fgraph = nullptr;
  int64_t fkey[7] = {-1, -1, -1, -1, -1, -1, 0};  // last entry: kernels in the graph
  cudaGraphExec_t sgraph = nullptr;
  int64_t skey[8] = {-1, -1, -1, -1, -1, -1, -1, 0};
  bool graphs = true;
  struct Rec {
    int cls;
    cudaEvent_t a, b;
  };
  std::vector<Rec> pending;
  std::vector<cudaEvent_t> pool;
  double prof_ms[KM_PROF_COUNT] = {};
  int64_t prof_n[KM_PROF_COUNT] = {};
};

namespace km {
// Handles of the batch and serving pools (one stream each, many at once) keep one CTA per node.
// The mixed form runs its leaf stage on the tensor cores unless KM_LEAF_TC=0 (the float-pair
// CUDA-core kernels, kept for comparison and for leaves above 1024 points).
bool leaf_tc_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("KM_LEAF_TC");
    return !(e && e[0] == '0');
  }();
  return on;
}

void set_node_cluster_max(km_handle* h, int v) {
  if (h) h->node_cluster_max = v < 1 ? 1 : v;
}
}  // namespace km

namespace {

constexpr int kLogdetBlocks = 256;

int fail(km_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_fail(km_handle* h, cudaError_t e, const char* where) {
  return fail(h, KM_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define KM_CUDA(h, call)                                  \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

int64_t device_budget(km_handle* h) {
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return INT64_MAX;
  const double f = h->cfg.hbm_budget_fraction > 0 ? h->cfg.hbm_budget_fraction : 0.8;
  return (int64_t)(f * (double)tot);
}

template <typename T>
int dalloc(km_handle* h, T** p, int64_t count) {
  const size_t bytes = (size_t)std::max<int64_t>(count, 1) * sizeof(T);
  if (h->bytes + (int64_t)bytes > device_budget(h))
    return fail(h, KM_ERR_OOM, "device memory budget exceeded");
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(h, KM_ERR_OOM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  h->allocs.push_back({q, bytes});
  h->alloc_epoch += 1;
  h->bytes += (int64_t)bytes;
  *p = (T*)q;
  return KM_OK;
}

void dfree(km_handle* h, void* p) {
  if (!p) return;
  for (size_t i = 0; i < h->allocs.size(); ++i) {
    if (h->allocs[i].first == p) {
      cudaFree(p);
      h->bytes -= (int64_t)h->allocs[i].second;
      h->allocs.erase(h->allocs.begin() + i);
      h->alloc_epoch += 1;
      return;
    }
  }
}

// Capacity-based allocation: keeps *p when its allocation already holds `count` elements, so a
// handle that serves problems of varying size reallocates only when a larger one arrives.
template <typename T>
int grow(km_handle* h, T** p, int64_t count) {
  const size_t bytes = (size_t)std::max<int64_t>(count, 1) * sizeof(T);
  if (*p) {
    for (auto& a : h->allocs)
      if (a.first == (void*)*p) {
        if (a.second >= bytes) return KM_OK;
        break;
      }
    dfree(h, *p);
    *p = nullptr;
  }
  return dalloc(h, p, count);
}

void free_problem(km_handle* h) {
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& a : h->allocs) cudaFree(a.first);
  h->allocs.clear();
  h->bytes = 0;
  h->d_pts = h->d_lnd = h->d_K = h->d_Lf = h->d_Phi = h->d_Q = h->d_tauleaf = h->d_R = nullptr;
  h->d_pts3 = h->d_lnd3 = nullptr;
  h->d_S = h->d_Sc = h->d_SinvT = h->d_SinvTf = h->d_Ct = h->d_L22 = h->d_Eref = h->d_Etau = nullptr;
  h->d_L22i = h->d_E = h->d_NT = nullptr;
  h->d_lcscr = nullptr;
  h->d_lndidx = nullptr;
  h->d_info = nullptr;
  h->d_partial = h->d_scalar = nullptr;
  h->d_VP = h->d_VG = h->d_VD = nullptr;
  h->vcap = 0;
  h->d_X = h->d_Y = nullptr;
  h->xcap = 0;
  h->blk.clear();
  h->brank.clear();
  h->lvoff.clear();
  h->gfoff.clear();
  h->d_blk = nullptr;
  h->d_panels = nullptr;
  h->d_flags = nullptr;
  h->d_piv = h->d_brank = h->d_bstatus = nullptr;
  h->d_R12 = h->d_CL = nullptr;
  h->d_gnodes = nullptr;
  h->d_gsolve = h->d_gfact = nullptr;
  h->gnodes_h.clear();
  h->gsolve_h.clear();
  h->gfact_h.clear();
  h->d_gz = nullptr;
  h->d_pqg = nullptr;
  h->d_pdesc = nullptr;
  h->d_ldesc = nullptr;
  h->nldesc = 0;
  h->gmaxr = 0;
  h->d_gpartial = nullptr;
  h->d_pqs = nullptr;
  h->d_acascr = nullptr;
  h->dk_param = -1;
  h->d_dK = h->d_dPhi = h->d_Sj = h->d_GP = h->d_GG = h->d_T = h->d_U = h->d_dots = h->d_A = nullptr;
  h->d_dKf = h->d_dPhif = h->d_Phif = nullptr;
  h->d_Sinv = h->d_SinvF = h->d_M2 = h->d_M2F = h->d_Mtmp = h->d_GB = nullptr;
  h->gcap = h->tcap = 0;
  h->d_res = h->d_rdots = nullptr;
  h->d_bkeep = nullptr;
  h->d_dPhi2 = h->d_Sj3 = h->d_Sj3F = h->d_VP4 = h->d_gpart = nullptr;
  h->rcap = 0;
  h->d2_pair = -1;
  h->d_hPhi3 = h->d_hD2 = h->d_hS = h->d_hT = h->d_hP = h->d_hG = h->d_hA = h->d_hY = h->d_hdots = nullptr;
  h->hcap = 0;
  h->assembled = h->factorized = false;
}

int check_launch(km_handle* h, const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, where);
  return KM_OK;
}

cudaEvent_t pool_event(km_handle* h) {
  if (!h->pool.empty()) {
    cudaEvent_t e = h->pool.back();
    h->pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Resolves the pending profiler records (their events have completed after a sync).
void prof_resolve(km_handle* h) {
  for (auto& r : h->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      h->prof_ms[r.cls] += ms;
      h->prof_n[r.cls] += 1;
    }
    h->pool.push_back(r.a);
    h->pool.push_back(r.b);
  }
  h->pending.clear();
  cudaGetLastError();
}

// Runs one kernel launch `f`, counting it and, when profiling, bracketing it with events.
template <typename F>
bool run_launch(km_handle* h, int cls, F&& f) {
  h->stats.kernel_launches += 1;
  if (!h->prof) return f();
  cudaEvent_t a = pool_event(h), b = pool_event(h);
  cudaEventRecord(a, h->stream);
  const bool ok = f();
  cudaEventRecord(b, h->stream);
  h->pending.push_back({cls, a, b});
  return ok;
}
#define KL(h, cls, expr) run_launch(h, cls, [&]() -> bool { return (expr); })
#define KLV(h, cls, expr) run_launch(h, cls, [&]() -> bool { expr; return true; })

int sync(km_handle* h, const char* where) {
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, where);
  if (h->prof) prof_resolve(h);
  return KM_OK;
}

void timer_start(km_handle* h) { cudaEventRecord(h->ev0, h->stream); }
double timer_stop(km_handle* h) {
  cudaEventRecord(h->ev1, h->stream);
  cudaEventSynchronize(h->ev1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  return ms;
}

int ensure_vec(km_handle* h, int64_t k) {
  if (k <= h->vcap) return KM_OK;
  h->vcap = 0;
  const int64_t slots = h->tree.nleaf + h->tree.nnode;
  int rc;
  if ((rc = grow(h, &h->d_VP, slots * h->r * k)) != KM_OK) return rc;
  if ((rc = grow(h, &h->d_VG, slots * h->r * k)) != KM_OK) return rc;
  if ((rc = grow(h, &h->d_VD, std::max<int64_t>(h->tree.nnode, 1) * 2 * h->r * k)) != KM_OK) return rc;
  h->vcap = k;
  return KM_OK;
}

int ensure_xy(km_handle* h, int64_t k) {
  if (k <= h->xcap) return KM_OK;
  h->xcap = 0;
  int rc;
  if ((rc = grow(h, &h->d_X, h->tree.n * k)) != KM_OK) return rc;
  if ((rc = grow(h, &h->d_Y, h->tree.n * k)) != KM_OK) return rc;
  h->xcap = k;
  return KM_OK;
}

NodeMatsH node_mats(km_handle* h) {
  const int64_t blk = std::max<int64_t>(h->tree.nnode, 1) * h->r * h->r;
  NodeMatsH nm{h->d_Ct, h->d_L22, h->d_L22i, h->d_E, h->r};
  nm.CtT = h->d_NT;
  nm.L22T = h->d_NT + blk;
  nm.L22iT = h->d_NT + 2 * blk;
  nm.ET = h->d_NT + 3 * blk;
  return nm;
}

// ---- factor sweeps on a device block X (n x k, ld = n), in place ---------------------------

// ---- general (ACA) path -------------------------------------------------------------------

// Nodes at least this large (rows of both children) apply their factor through library GEMMs:
// k_gapply gives one warp per (node, column), which serialises the O(size x rank) projections
// of the top levels on a few SMs.
constexpr int64_t kGapplyBig = 16384;
// Panels with at least this many rows apply their block reflectors as library GEMMs (one CTA per
// 8-column tile over all rows leaves most SMs idle on the few tall panels of the top levels).
constexpr int64_t kPanelBig = 16384;

// Applies the node factors of items [a, b) of a level (host list hl, device list dl): k_gapply for
// the small nodes, and for every large node Z = Q' x (DGEMM), the r x r part (k_gsmall), then
// y -= / += Q G (DGEMM).  Modes as in k_gapply: 0 W^{-1}, 1 W'^{-1}, 2 W, 3 W', 4 pre-factor
// product (Q1 = V rows c1, Q2 = U rows c2; y1 += V U' x2, y2 += U V' x1).
static int run_gapply(km_handle* h, const std::vector<GApplyItem>& hl, GApplyItem* dl, int64_t a, int64_t b,
                      int maxcols, int mode, double* X, const double* Xin, int64_t ldX, int kX) {
  cudaStream_t st = h->stream;
  if (b <= a) return KM_OK;
  KLV(h, KM_PROF_SWEEP, launch_gapply(dl + a, (int)(b - a), h->d_gnodes, h->gmaxr, maxcols, mode, X, Xin, ldX, kX, st));
  int64_t need = 0, split = 0;
  for (int64_t q = a; q < b; ++q)
    if (hl[q].big) {
      const GNodeDesc& N = h->gnodes_h[hl[q].node];
      const int nc = hl[q].base ? hl[q].ncols : kX;
      need = std::max<int64_t>(need, 4 * (int64_t)N.r * nc);
      split = std::max(split, std::max(dgemm_scratch(1, N.r, nc, N.s1), dgemm_scratch(1, N.r, nc, N.s2)));
    }
  if (need == 0) return KM_OK;
  int rc;
  if ((rc = grow(h, &h->d_gz, need + split)) != KM_OK) return rc;
  const double one = 1.0, mone = -1.0;
  for (int64_t q = a; q < b; ++q) {
    const GApplyItem& I = hl[q];
    if (!I.big) continue;
    const GNodeDesc& N = h->gnodes_h[I.node];
    const int r = N.r;
    double* base = I.base ? I.base : X;
    const int64_t ld = I.base ? I.ld : ldX;
    const int nc = I.base ? I.ncols : kX;
    if (r <= 0 || nc <= 0) continue;
    double* y1 = base + I.off1;
    double* y2 = base + I.off2;
    const double* x1 = (mode == 4) ? Xin + I.off1 : y1;
    const double* x2 = (mode == 4) ? Xin + I.off2 : y2;
    double* Z1 = h->d_gz;
    double* Z2 = Z1 + (int64_t)r * nc;
    double* G1 = Z2 + (int64_t)r * nc;
    double* G2 = G1 + (int64_t)r * nc;
    const int64_t s1 = N.s1, s2 = N.s2;
    double* spl = G2 + (int64_t)r * nc;  // partial products of the split Q' x reductions
    auto gemm_t = [&](const double* Q, int64_t s, const double* x, double* Z) {  // Z = Q' x
      launch_dgemm(1, r, nc, s, 1.0, Q, s, x, ld, 0.0, Z, r, spl, split, st);
    };
    auto gemm_n = [&](const double* Q, int64_t s, const double* G, double* y, const double* alpha) {  // y += a Q G
      launch_dgemm(0, s, nc, r, *alpha, Q, s, G, r, 1.0, y, ld, nullptr, 0, st);
    };
    const GNodeDesc* dN = h->d_gnodes + I.node;
    KLV(h, KM_PROF_SWEEP, {
      if (mode == 4) {
        gemm_t(N.Q2, s2, x2, Z1);  // U' x2
        gemm_t(N.Q1, s1, x1, Z2);  // V' x1
        gemm_n(N.Q1, s1, Z1, y1, &one);
        gemm_n(N.Q2, s2, Z2, y2, &one);
      } else {
        if (mode == 0 || mode == 2) gemm_t(N.Q1, s1, x1, Z1);
        gemm_t(N.Q2, s2, x2, Z2);
        launch_gsmall(dN, mode, Z1, Z2, G1, G2, r, nc, st);
        if (mode == 1 || mode == 3) gemm_n(N.Q1, s1, G1, y1, mode == 1 ? &mone : &one);
        gemm_n(N.Q2, s2, G2, y2, (mode == 0 || mode == 1) ? &mone : &one);
      }
    });
  }
  return check_launch(h, "factor application");
}

int general_fwd(km_handle* h, double* X, int k) {  // X <- W^{-1} X
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri<double>(h->d_Lf, t, 0, X, 1, t.n, 0, X, 1, t.n, 0, k, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular solve kernel");
  for (int l = 1; l <= t.L; ++l) {
    const int64_t a = h->lvoff[l], b = h->lvoff[l + 1];
    int rc;
    if ((rc = run_gapply(h, h->gsolve_h, h->d_gsolve, a, b, k, 0, X, X, t.n, k)) != KM_OK) return rc;
  }
  return check_launch(h, "general fwd");
}

int general_bwd(km_handle* h, double* X, int k) {  // X <- W'^{-1} X
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  for (int l = t.L; l >= 1; --l) {
    const int64_t a = h->lvoff[l], b = h->lvoff[l + 1];
    int rc;
    if ((rc = run_gapply(h, h->gsolve_h, h->d_gsolve, a, b, k, 1, X, X, t.n, k)) != KM_OK) return rc;
  }
  if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri<double>(h->d_Lf, t, 1, X, 1, t.n, 0, X, 1, t.n, 0, k, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular solve kernel");
  return check_launch(h, "general bwd");
}

int general_mul(km_handle* h, double* X, int k) {  // X <- W X
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  for (int l = t.L; l >= 1; --l) {
    const int64_t a = h->lvoff[l], b = h->lvoff[l + 1];
    int rc;
    if ((rc = run_gapply(h, h->gsolve_h, h->d_gsolve, a, b, k, 2, X, X, t.n, k)) != KM_OK) return rc;
  }
  if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri<double>(h->d_Lf, t, 2, X, 1, t.n, 0, X, 1, t.n, 0, k, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular kernel");
  return check_launch(h, "general mul");
}

int general_mul_t(km_handle* h, double* X, int k) {  // X <- W' X
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri<double>(h->d_Lf, t, 3, X, 1, t.n, 0, X, 1, t.n, 0, k, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular kernel");
  for (int l = 1; l <= t.L; ++l) {
    const int64_t a = h->lvoff[l], b = h->lvoff[l + 1];
    int rc;
    if ((rc = run_gapply(h, h->gsolve_h, h->d_gsolve, a, b, k, 3, X, X, t.n, k)) != KM_OK) return rc;
  }
  return check_launch(h, "general mul_t");
}

// Y = K X before factorisation: leaf products, then V (U' x) and U (V' x) block by block
// (src/HODLR/src/baseoverloads.jl:152-169), level by level because levels share rows.
int general_matvec(km_handle* h, const double* X, double* Y, int k) {
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_nys_apply(h->d_K, nullptr, nullptr, 0, t, X, t.n, nullptr, Y, t.n, k, st));
  for (int l = 1; l <= t.L; ++l) {
    const int64_t a = h->lvoff[l], b = h->lvoff[l + 1];
    int rc;
    if ((rc = run_gapply(h, h->gsolve_h, h->d_gsolve, a, b, k, 4, Y, X, t.n, k)) != KM_OK) return rc;
  }
  return check_launch(h, "general matvec");
}

template <typename T>
T* P(double* p) {
  return reinterpret_cast<T*>(p);
}

// The block solve re-reads a leaf's factor for every chunk of 4 right-hand sides; from 32
// columns on (the probe blocks of the gradient) the substitution kernel's wider chunks win.
static bool use_tri_blk(const km_handle* h, int64_t k) { return h->leaf_tc && k < 32; }

// Leaf solve L x = b (op 0) or L' x = b (op 1) on k columns in place: by 64-row blocks with the
// diagonal-block inverses the tensor-core leaf stage keeps, else by substitution.
template <typename T>
static bool leaf_solve(km_handle* h, int op, T* X, int k) {
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  if constexpr (std::is_same<T, ff>::value) {
    if (use_tri_blk(h, k)) return KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri_blk(P<ff>(h->d_Lf), t, op, X, t.n, k, st));
  }
  return KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri<T>(P<T>(h->d_Lf), t, op, X, 1, t.n, 0, X, 1, t.n, 0, k, st));
}

template <typename T>
int nested_fwd_t(km_handle* h, T* X, int k) {  // X <- W^{-1} X
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  if (!leaf_solve<T>(h, 0, X, k))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular solve kernel");
  if (t.L == 0) return check_launch(h, "fwd");
  NodeMatsH nm = node_mats(h);
  KLV(h, KM_PROF_LEAF_REFL, launch_leaf_proj<T>(P<T>(h->d_Q), P<T>(h->d_tauleaf), h->r, t, X, t.n, P<T>(h->d_VP), k, st));
  for (int l = 1; l <= t.L; ++l) KLV(h, KM_PROF_SWEEP, launch_up<T>(t, nm, l, P<T>(h->d_VP), P<T>(h->d_VD), k, UP_FWD_, st));
  for (int l = t.L; l >= 1; --l) KLV(h, KM_PROF_SWEEP, launch_down<T>(t, nm, l, P<T>(h->d_VP), P<T>(h->d_VG), P<T>(h->d_VD), k, DN_FWD_, st));
  KLV(h, KM_PROF_LEAF_REFL, launch_leaf_expand<T>(P<T>(h->d_Q), P<T>(h->d_tauleaf), h->r, t, P<T>(h->d_VG), X, t.n, k, -1.0, st));
  return check_launch(h, "fwd");
}

// after_fwd: X comes straight from nested_fwd_t, whose leaf slots still hold z = Q'x (VP) and
// the coefficients g it expanded (VG, x <- x - Q g); with Q'Q = I the new projections are
// z - g, so the projection pass over the leaves is skipped (leaves of at least r rows, where
// the leaf bases have r orthonormal columns).
template <typename T>
int nested_bwd_t(km_handle* h, T* X, int k, bool after_fwd = false) {  // X <- W'^{-1} X
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  if (t.L > 0) {
    NodeMatsH nm = node_mats(h);
    if (after_fwd && t.m0 >= h->r)
      KLV(h, KM_PROF_LEAF_REFL, launch_slot_sub<T>(P<T>(h->d_VP), P<T>(h->d_VG), t.nleaf * (int64_t)k * h->r, st));
    else
      KLV(h, KM_PROF_LEAF_REFL, launch_leaf_proj<T>(P<T>(h->d_Q), P<T>(h->d_tauleaf), h->r, t, X, t.n, P<T>(h->d_VP), k, st));
    for (int l = 1; l < t.L; ++l) KLV(h, KM_PROF_SWEEP, launch_up<T>(t, nm, l, P<T>(h->d_VP), P<T>(h->d_VD), k, UP_PROJ_, st));
    for (int l = t.L; l >= 1; --l) KLV(h, KM_PROF_SWEEP, launch_down<T>(t, nm, l, P<T>(h->d_VP), P<T>(h->d_VG), P<T>(h->d_VD), k, DN_BWD_, st));
    KLV(h, KM_PROF_LEAF_REFL, launch_leaf_expand<T>(P<T>(h->d_Q), P<T>(h->d_tauleaf), h->r, t, P<T>(h->d_VG), X, t.n, k, -1.0, st));
  }
  if (!leaf_solve<T>(h, 1, X, k)) return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular solve kernel");
  return check_launch(h, "bwd");
}

template <typename T>
int nested_mul_t_(km_handle* h, T* X, int k) {  // X <- W X
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  if (t.L > 0) {
    NodeMatsH nm = node_mats(h);
    KLV(h, KM_PROF_LEAF_REFL, launch_leaf_proj<T>(P<T>(h->d_Q), P<T>(h->d_tauleaf), h->r, t, X, t.n, P<T>(h->d_VP), k, st));
    for (int l = 1; l < t.L; ++l) KLV(h, KM_PROF_SWEEP, launch_up<T>(t, nm, l, P<T>(h->d_VP), P<T>(h->d_VD), k, UP_PROJ_, st));
    for (int l = t.L; l >= 1; --l) KLV(h, KM_PROF_SWEEP, launch_down<T>(t, nm, l, P<T>(h->d_VP), P<T>(h->d_VG), P<T>(h->d_VD), k, DN_MUL_, st));
    KLV(h, KM_PROF_LEAF_REFL, launch_leaf_expand<T>(P<T>(h->d_Q), P<T>(h->d_tauleaf), h->r, t, P<T>(h->d_VG), X, t.n, k, 1.0, st));
  }
  if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri<T>(P<T>(h->d_Lf), t, 2, X, 1, t.n, 0, X, 1, t.n, 0, k, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular kernel");
  return check_launch(h, "mul");
}

template <typename T>
int nested_mult_t(km_handle* h, T* X, int k) {  // X <- W' X
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri<T>(P<T>(h->d_Lf), t, 3, X, 1, t.n, 0, X, 1, t.n, 0, k, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular kernel");
  if (t.L == 0) return check_launch(h, "mul_t");
  NodeMatsH nm = node_mats(h);
  KLV(h, KM_PROF_LEAF_REFL, launch_leaf_proj<T>(P<T>(h->d_Q), P<T>(h->d_tauleaf), h->r, t, X, t.n, P<T>(h->d_VP), k, st));
  for (int l = 1; l <= t.L; ++l) KLV(h, KM_PROF_SWEEP, launch_up<T>(t, nm, l, P<T>(h->d_VP), P<T>(h->d_VD), k, UP_MULT_, st));
  for (int l = t.L; l >= 1; --l) KLV(h, KM_PROF_SWEEP, launch_down<T>(t, nm, l, P<T>(h->d_VP), P<T>(h->d_VG), P<T>(h->d_VD), k, DN_MULT_, st));
  KLV(h, KM_PROF_LEAF_REFL, launch_leaf_expand<T>(P<T>(h->d_Q), P<T>(h->d_tauleaf), h->r, t, P<T>(h->d_VG), X, t.n, k, 1.0, st));
  return check_launch(h, "mul_t");
}

// Dispatch on the method and the precision.  In the mixed form the factor holds float pairs and
// the block X (n x k, ld n) is converted in place around the float-pair kernels.
int nested_fwd(km_handle* h, double* X, int k) {
  if (h->method == KM_METHOD_ACA) return general_fwd(h, X, k);
  if (!h->mixed) return nested_fwd_t<double>(h, X, k);
  ff* Xf = reinterpret_cast<ff*>(X);
  KLV(h, KM_PROF_OTHER, launch_to_ff(X, Xf, h->tree.n * k, h->stream));
  const int rc = nested_fwd_t<ff>(h, Xf, k);
  KLV(h, KM_PROF_OTHER, launch_from_ff(Xf, X, h->tree.n * k, h->stream));
  return rc;
}

int nested_bwd(km_handle* h, double* X, int k) {
  if (h->method == KM_METHOD_ACA) return general_bwd(h, X, k);
  if (!h->mixed) return nested_bwd_t<double>(h, X, k);
  ff* Xf = reinterpret_cast<ff*>(X);
  KLV(h, KM_PROF_OTHER, launch_to_ff(X, Xf, h->tree.n * k, h->stream));
  const int rc = nested_bwd_t<ff>(h, Xf, k);
  KLV(h, KM_PROF_OTHER, launch_from_ff(Xf, X, h->tree.n * k, h->stream));
  return rc;
}

// K^{-1} X = W'^{-1} W^{-1} X with one conversion pair in the mixed form
int nested_solve(km_handle* h, double* X, int k) {
  if (h->method == KM_METHOD_ACA) {
    const int rc = general_fwd(h, X, k);
    return rc != KM_OK ? rc : general_bwd(h, X, k);
  }
  if (!h->mixed) {
    const int rc = nested_fwd_t<double>(h, X, k);
    return rc != KM_OK ? rc : nested_bwd_t<double>(h, X, k, true);
  }
  ff* Xf = reinterpret_cast<ff*>(X);
  KLV(h, KM_PROF_OTHER, launch_to_ff(X, Xf, h->tree.n * k, h->stream));
  int rc = nested_fwd_t<ff>(h, Xf, k);
  if (rc == KM_OK) rc = nested_bwd_t<ff>(h, Xf, k, true);
  KLV(h, KM_PROF_OTHER, launch_from_ff(Xf, X, h->tree.n * k, h->stream));
  return rc;
}

int nested_mul(km_handle* h, double* X, int k) {
  if (h->method == KM_METHOD_ACA) return general_mul(h, X, k);
  if (!h->mixed) return nested_mul_t_<double>(h, X, k);
  ff* Xf = reinterpret_cast<ff*>(X);
  KLV(h, KM_PROF_OTHER, launch_to_ff(X, Xf, h->tree.n * k, h->stream));
  const int rc = nested_mul_t_<ff>(h, Xf, k);
  KLV(h, KM_PROF_OTHER, launch_from_ff(Xf, X, h->tree.n * k, h->stream));
  return rc;
}

int nested_mul_t(km_handle* h, double* X, int k) {
  if (h->method == KM_METHOD_ACA) return general_mul_t(h, X, k);
  if (!h->mixed) return nested_mult_t<double>(h, X, k);
  ff* Xf = reinterpret_cast<ff*>(X);
  KLV(h, KM_PROF_OTHER, launch_to_ff(X, Xf, h->tree.n * k, h->stream));
  const int rc = nested_mult_t<ff>(h, Xf, k);
  KLV(h, KM_PROF_OTHER, launch_from_ff(Xf, X, h->tree.n * k, h->stream));
  return rc;
}

// Y = K X before factorisation (Nystrom blocks)
int nystrom_matvec(km_handle* h, const double* X, double* Y, int k) {
  if (h->method == KM_METHOD_ACA) return general_matvec(h, X, Y, k);
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  if (t.L > 0) {
    KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_phiT(h->d_Phi, h->r, t, X, t.n, h->d_VP, k, st));
    KLV(h, KM_PROF_SWEEP, launch_nys_sums(h->d_VP, h->d_VG, t.nleaf, h->r, k, st));
  } else {
    cudaMemsetAsync(h->d_VG, 0, sizeof(double) * h->r * k, st);
  }
  KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_nys_apply(h->d_K, h->d_Phi, h->d_Sc, h->r, t, X, t.n, h->d_VG, Y, t.n, k, st));
  return check_launch(h, "matvec");
}


// Mixed form: FP64 iterative refinement x += K~^{-1} (b - K x), with the FP64 Nystrom HODLR
// product as the residual operator (it keeps the FP64 leaves and landmark columns) and the
// float-pair factor K~ as the preconditioner; stops at ||b - Kx||_F <= refine_tol ||b||_F.
// The caller provides the buffers: res (n x k doubles), rdots (2k doubles, device) and hdots
// (2k doubles, host).  d_b must not alias d_x.
int refine_with(km_handle* h, const double* d_b, double* d_x, int k, double* res, double* rdots, double* hdots) {
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  int rc;
  KLV(h, KM_PROF_OTHER, launch_col_dots(d_b, t.n, d_b, t.n, t.n, k, rdots + k, st));
  int it = 0;
  double relres = 0.0;
  for (;;) {
    if ((rc = nystrom_matvec(h, d_x, res, k)) != KM_OK) return rc;
    KLV(h, KM_PROF_OTHER, launch_axpby(res, d_b, 1.0, -1.0, t.n * k, st));  // res = b - K x
    KLV(h, KM_PROF_OTHER, launch_col_dots(res, t.n, res, t.n, t.n, k, rdots, st));
    KM_CUDA(h, cudaMemcpyAsync(hdots, rdots, sizeof(double) * 2 * k, cudaMemcpyDeviceToHost, st));
    if ((rc = sync(h, "refine")) != KM_OK) return rc;
    double rr = 0.0, bb = 0.0;
    for (int c = 0; c < k; ++c) {
      rr += hdots[c];
      bb += hdots[k + c];
    }
    relres = bb > 0.0 ? std::sqrt(rr / bb) : 0.0;
    if (relres <= h->cfg.refine_tol || it >= h->cfg.refine_max_iter) break;
    if ((rc = nested_solve(h, res, k)) != KM_OK) return rc;
    KLV(h, KM_PROF_OTHER, launch_axpby(d_x, res, 1.0, 1.0, t.n * k, st));  // x += d
    ++it;
  }
  h->stats.refine_iterations = it;
  h->stats.refine_residual = relres;
  return KM_OK;
}

// Refinement on the handle's own workspace.  d_b_saved is a copy of the right-hand sides when
// the solve ran in place (d_b == d_x), else d_b itself.
int refine(km_handle* h, const double* d_b, double* d_x, int k) {
  int rc;
  if (k > h->rcap) {
    h->rcap = 0;
    if ((rc = grow(h, &h->d_res, 2 * h->tree.n * k)) || (rc = grow(h, &h->d_rdots, 2 * k))) return rc;
    h->rcap = k;
  }
  std::vector<double> dots(2 * k);
  return refine_with(h, d_b, d_x, k, h->d_res, h->d_rdots, dots.data());
}

// Side stream: forms explicit leaf bases and node solve operators concurrently with the node
// levels on the main stream (they are needed only by solves and products).
void side_begin(km_handle* h) {
  cudaEventRecord(h->sev[0], h->stream);
  cudaStreamWaitEvent(h->side, h->sev[0], 0);
  h->stats.kernel_launches += 1;
}
void side_level(km_handle* h, int l) {
  cudaEventRecord(h->sev[l], h->stream);
  cudaStreamWaitEvent(h->side, h->sev[l], 0);
  h->stats.kernel_launches += 1;
}
void side_end(km_handle* h) {
  cudaEventRecord(h->sev[kMaxLevels + 2], h->side);
  cudaStreamWaitEvent(h->stream, h->sev[kMaxLevels + 2], 0);
}

// Enqueues the copy of d_info[0 .. count) into the pinned h_info on the handle's stream; the
// words are valid after the next synchronisation of that stream.
// The buffer starts at 8192 words (trees of up to 4096 leaves) and doubles: freeing pinned memory
// synchronises the device, which would stall the other handles of a pool, so it regrows rarely.
int fetch_info_async(km_handle* h, int64_t count) {
  if (count > h->h_info_cap) {
    const int64_t cap = std::max<int64_t>(count, std::max<int64_t>(8192, 2 * h->h_info_cap));
    if (h->h_info) cudaFreeHost(h->h_info);
    h->h_info = nullptr;
    h->h_info_cap = 0;
    if (cudaMallocHost(&h->h_info, sizeof(int) * (size_t)cap) != cudaSuccess) {
      cudaGetLastError();
      h->h_info = nullptr;
      return fail(h, KM_ERR_OOM, "pinned host buffer for the pivot status");
    }
    h->h_info_cap = cap;
  }
  KM_CUDA(h, cudaMemcpyAsync(h->h_info, h->d_info, sizeof(int) * count, cudaMemcpyDeviceToHost, h->stream));
  return KM_OK;
}

// The leaf pivot status in info[0 .. count): PosDefException for the first failing leaf.
int check_info_words(km_handle* h, const int* info, int64_t count, const char* what) {
  for (int64_t i = 0; i < count; ++i) {
    if (info[i] < 0) return fail(h, KM_ERR_TIMEOUT, "a bounded wait of the tensor-core leaf update ran out");
    if (info[i] != 0) {
      char buf[160];
      snprintf(buf, sizeof buf, "PosDefException: %s %lld is not positive definite (pivot %d)",
               what, (long long)i, info[i]);
      return fail(h, KM_ERR_NOT_SPD, buf);
    }
  }
  return KM_OK;
}

int check_info(km_handle* h, int64_t count, const char* what) {
  std::vector<int> info(count);
  KM_CUDA(h, cudaMemcpy(info.data(), h->d_info, sizeof(int) * count, cudaMemcpyDeviceToHost));
  return check_info_words(h, info.data(), count, what);
}

// Y = dK_j X for the exact derivative of the Nystrom HODLR in parameter j (device pointers).
int derivative_apply(km_handle* h, int j, const double* X, double* Y, int k) {
  const Tree& t = h->tree;
  const int r = h->r;
  cudaStream_t st = h->stream;
  int rc;
  int64_t kbytes = 0;
  for (int64_t q = 0; q < t.nleaf; ++q) kbytes += t.leaf_size(q) * t.leaf_size(q);
  if (h->dk_param < 0) {
    if ((rc = grow(h, &h->d_dK, kbytes)) || (rc = grow(h, &h->d_dPhi, t.n * r)) || (rc = grow(h, &h->d_Sj, r * r)))
      return rc;
    if (h->mixed) {
      // float-pair copies for the derivative products of the mixed form (FP32 pipe), and the
      // explicit S^{-1} = Sc^{-T} Sc^{-1} that replaces the per-column landmark solves
      if ((rc = grow(h, &h->d_dKf, kbytes)) || (rc = grow(h, &h->d_dPhif, t.n * r)) ||
          (rc = grow(h, &h->d_Phif, t.n * r)) || (rc = grow(h, &h->d_Sinv, r * r)) ||
          (rc = grow(h, &h->d_SinvF, r * r)) || (rc = grow(h, &h->d_M2, r * r)) || (rc = grow(h, &h->d_M2F, r * r)) ||
          (rc = grow(h, &h->d_Mtmp, r * r)))
        return rc;
      KLV(h, KM_PROF_OTHER, launch_to_ff(h->d_Phi, P<ff>(h->d_Phif), t.n * r, st));
      KLV(h, KM_PROF_OTHER, launch_small_gemm(h->d_SinvT, h->d_SinvT, r, 1, h->d_Sinv, st));
      KLV(h, KM_PROF_OTHER, launch_to_ff(h->d_Sinv, P<ff>(h->d_SinvF), (int64_t)r * r, st));
    }
  }
  if (k > h->gcap) {
    h->gcap = 0;
    const int64_t slots = t.nleaf + t.nnode;
    if ((rc = grow(h, &h->d_GP, slots * 2 * r * k)) || (rc = grow(h, &h->d_GG, slots * 2 * r * k))) return rc;
    h->gcap = k;
  }
  if (h->dk_param != j) {
    // DerivativeHODLR (constructor.jl:66-95): dK leaves, dK(X, P) and Sj = dK(P, P)
    KLV(h, KM_PROF_EVAL, launch_eval_leaves(h->d_pts, t, h->kp, j, h->d_dK, st, h->mixed));
    KLV(h, KM_PROF_EVAL, launch_eval_phi(h->d_pts, h->d_lnd, r, t, h->kp, j, h->d_dPhi, st, h->mixed));
    KLV(h, KM_PROF_EVAL, launch_eval_dense(h->d_lnd, r, h->d_lnd, r, h->kp, j, h->d_Sj, r, st));
    if (h->mixed) {
      KLV(h, KM_PROF_OTHER, launch_to_ff(h->d_dK, P<ff>(h->d_dKf), kbytes, st));
      KLV(h, KM_PROF_OTHER, launch_to_ff(h->d_dPhi, P<ff>(h->d_dPhif), t.n * r, st));
      // M2 = S^{-1} Sj S^{-1}
      KLV(h, KM_PROF_OTHER, launch_small_gemm(h->d_Sj, h->d_Sinv, r, 0, h->d_Mtmp, st));
      KLV(h, KM_PROF_OTHER, launch_small_gemm(h->d_Sinv, h->d_Mtmp, r, 0, h->d_M2, st));
      KLV(h, KM_PROF_OTHER, launch_to_ff(h->d_M2, P<ff>(h->d_M2F), (int64_t)r * r, st));
    }
    h->dk_param = j;
  }
  if (t.L > 0) {
    if (h->mixed)
      KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_dphiT<ff>(P<ff>(h->d_Phif), P<ff>(h->d_dPhif), r, t, X, t.n, h->d_GP, k, st));
    else
      KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_dphiT<double>(h->d_Phi, h->d_dPhi, r, t, X, t.n, h->d_GP, k, st));
    KLV(h, KM_PROF_SWEEP, launch_nys_sums(h->d_GP, h->d_GG, t.nleaf, 2 * r, k, st));
  } else {
    KM_CUDA(h, cudaMemsetAsync(h->d_GG, 0, sizeof(double) * 2 * r * k, st));
  }
  if (h->mixed) {
    if ((rc = grow(h, &h->d_GB, t.nleaf * 2 * r * k))) return rc;
    KLV(h, KM_PROF_LEAF_APPLY, launch_dbeta<ff>(P<ff>(h->d_SinvF), P<ff>(h->d_M2F), r, h->d_GG, t.nleaf * (int64_t)k,
                                                P<ff>(h->d_GB), st));
    KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_dnys_apply<ff>(P<ff>(h->d_dKf), P<ff>(h->d_Phif), P<ff>(h->d_dPhif), h->d_Sc,
                                                          h->d_Sj, r, t, X, t.n, h->d_GG, Y, t.n, k, st,
                                                          P<ff>(h->d_GB)));
  }
  else
    KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_dnys_apply<double>(h->d_dK, h->d_Phi, h->d_dPhi, h->d_Sc, h->d_Sj, r, t, X,
                                                              t.n, h->d_GG, Y, t.n, k, st));
  return check_launch(h, "derivative");
}

// Y = D2_jk X (Deriv2mul, src/HODLR/src/utils.jl:157-177) for parameters j <= k: the dense
// second-derivative leaves plus the reference's block products SDBlock_mul / SDBlock_mul_t
// (utils.jl:110-155) of every non-leaf block, in the nested form of km_grad.cu (device pointers,
// FP64 in both precision forms; k columns).
int deriv2_apply(km_handle* h, int j, int k, const double* X, double* Y, int kc) {
  const Tree& t = h->tree;
  const int r = h->r, R = 4 * r;
  cudaStream_t st = h->stream;
  int rc;
  const int code = kD2Base + 3 * j + k;
  if (h->d2_pair != code) {
    int64_t kbytes = 0;
    for (int64_t q = 0; q < t.nleaf; ++q) kbytes += t.leaf_size(q) * t.leaf_size(q);
    const int64_t rr = (int64_t)r * r;
    if ((rc = grow(h, &h->d_hPhi3, 3 * t.n * r)) || (rc = grow(h, &h->d_hD2, kbytes)) ||
        (rc = grow(h, &h->d_hS, 12 * rr)) || (rc = grow(h, &h->d_hT, 2 * (int64_t)R * R)))
      return rc;
    double* Pj = h->d_hPhi3;
    double* Pk = Pj + t.n * r;
    double* Pjk = Pk + t.n * r;
    // SecondDerivativeLeaves / SecondDerivativeBlocks (constructor.jl:100-121) and the first
    // derivatives of the same blocks (constructor.jl:66-95)
    KLV(h, KM_PROF_EVAL, launch_eval_phi(h->d_pts, h->d_lnd, r, t, h->kp, j, Pj, st, false));
    KLV(h, KM_PROF_EVAL, launch_eval_phi(h->d_pts, h->d_lnd, r, t, h->kp, k, Pk, st, false));
    KLV(h, KM_PROF_EVAL, launch_eval_phi(h->d_pts, h->d_lnd, r, t, h->kp, code, Pjk, st, false));
    KLV(h, KM_PROF_EVAL, launch_eval_leaves(h->d_pts, t, h->kp, code, h->d_hD2, st, false));
    double* Sj = h->d_hS;
    double* Sk = Sj + rr;
    double* Sjk = Sk + rr;
    double* tA = Sjk + rr;
    double* tB = tA + rr;
    double* tC = tB + rr;
    double* M = tC + rr;  // A = S^{-1}, Bj, Bk, Bjk, Cjk, Ckj
    KLV(h, KM_PROF_EVAL, launch_eval_dense(h->d_lnd, r, h->d_lnd, r, h->kp, j, Sj, r, st));
    KLV(h, KM_PROF_EVAL, launch_eval_dense(h->d_lnd, r, h->d_lnd, r, h->kp, k, Sk, r, st));
    KLV(h, KM_PROF_EVAL, launch_eval_dense(h->d_lnd, r, h->d_lnd, r, h->kp, code, Sjk, r, st));
    KLV(h, KM_PROF_OTHER, launch_small_gemm(h->d_SinvT, h->d_SinvT, r, 1, M, st));  // S^{-1} = Sc^{-T} Sc^{-1}
    KLV(h, KM_PROF_OTHER, launch_small_gemm(Sj, M, r, 0, tA, st));
    KLV(h, KM_PROF_OTHER, launch_small_gemm(Sk, M, r, 0, tB, st));
    KLV(h, KM_PROF_OTHER, launch_small_gemm(Sjk, M, r, 0, tC, st));
    KLV(h, KM_PROF_OTHER, launch_small_gemm(M, tA, r, 0, M + rr, st));          // Bj = A Sj A
    KLV(h, KM_PROF_OTHER, launch_small_gemm(M, tB, r, 0, M + 2 * rr, st));      // Bk
    KLV(h, KM_PROF_OTHER, launch_small_gemm(M, tC, r, 0, M + 3 * rr, st));      // Bjk
    KLV(h, KM_PROF_OTHER, launch_small_gemm(M + rr, tB, r, 0, M + 4 * rr, st));  // Cjk = Bj Sk A
    KLV(h, KM_PROF_OTHER, launch_small_gemm(M + 2 * rr, tA, r, 0, M + 5 * rr, st));  // Ckj = Bk Sj A
    KLV(h, KM_PROF_OTHER, launch_d2_assemble(M, r, h->d_hT, h->d_hT + (int64_t)R * R, st));
    h->d2_pair = code;
  }
  if (kc > h->hcap) {
    h->hcap = 0;
    const int64_t slots = t.nleaf + t.nnode;
    if ((rc = grow(h, &h->d_hP, slots * R * kc)) || (rc = grow(h, &h->d_hG, slots * R * kc))) return rc;
    h->hcap = kc;
  }
  if (t.L > 0) {
    KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_phi4T(h->d_Phi, h->d_hPhi3, r, t, X, t.n, h->d_hP, kc, st));
    NodeMatsH nm4{nullptr, nullptr, nullptr, nullptr, R};
    for (int l = 1; l < t.L; ++l) KLV(h, KM_PROF_SWEEP, launch_up<double>(t, nm4, l, h->d_hP, nullptr, kc, UP_SUM_, st));
    for (int l = t.L; l >= 1; --l)
      KLV(h, KM_PROF_SWEEP, launch_d2_down(h->d_hT, h->d_hT + (int64_t)R * R, r, t, l, h->d_hP, h->d_hG, kc, st));
    KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_d2_apply(h->d_hD2, h->d_Phi, h->d_hPhi3, r, t, X, t.n, h->d_hG, Y, t.n,
                                                    kc, st));
  } else {
    KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_d2_apply(h->d_hD2, h->d_Phi, h->d_hPhi3, r, t, X, t.n, nullptr, Y, t.n,
                                                    kc, st));
  }
  return check_launch(h, "second derivative");
}

// Pairs whose second derivative vanishes identically (ZeroFunction in stoch_hessian): every
// pair with the nugget, and scale-scale for the Matern kernel (linear in the scale).
bool d2_zero(int kid, int j, int k) { return k == 2 || j == 2 || (kid == KM_KERNEL_MATERN32 && j == 0 && k == 0); }

bool finite3(const double* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

}  // namespace

// ---------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------
// Runs `body` (an asynchronous launch sequence on h->stream, possibly forking the side stream)
// through a CUDA graph when KM_GRAPHS is set in the environment: replays the cached graph when
// the key (all entries but the last) matches, else captures body into a new graph and launches
// it; the last key entry holds the number of kernels the graph launches, added to the launch
// count on each replay.  With profiling on the sequence runs directly, and a capture that fails
// falls back to direct launches.  Off by default: at n = 2^16, FixedLevel(8) the graphed
// factorisation and solve measured 2 % slower than direct launches (graph kernel nodes do not
// keep the side stream's lower priority).
template <size_t N, typename F>
static int run_graphed(km_handle* h, cudaGraphExec_t* cache, int64_t (&cached_key)[N], const int64_t (&key)[N - 1],
                       F&& body) {
  static const bool enabled = std::getenv("KM_GRAPHS") != nullptr;
  if (h->prof || !enabled || !h->graphs) return body();
  cudaStream_t st = h->stream;
  bool same = *cache != nullptr;
  for (size_t i = 0; i + 1 < N && same; ++i) same = cached_key[i] == key[i];
  if (same) {
    const cudaError_t e = cudaGraphLaunch(*cache, st);
    if (e == cudaSuccess) {
      h->stats.kernel_launches += cached_key[N - 1];
      return KM_OK;
    }
    cudaGetLastError();
  }
  if (*cache) {
    cudaGraphExecDestroy(*cache);
    *cache = nullptr;
  }
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
    cudaGetLastError();
    return body();
  }
  const int64_t launches0 = h->stats.kernel_launches;
  const int rc = body();
  const int64_t nk = h->stats.kernel_launches - launches0;
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(st, &g);
  if (rc != KM_OK) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return rc;
  }
  cudaGraphExec_t ex = nullptr;
  if (e != cudaSuccess || !g || cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    h->graphs = false;  // this handle's sequences do not capture: launch directly from now on
    h->stats.kernel_launches = launches0;
    return body();
  }
  cudaGraphDestroy(g);
  *cache = ex;
  for (size_t i = 0; i + 1 < N; ++i) cached_key[i] = key[i];
  cached_key[N - 1] = nk;
  if (cudaGraphLaunch(ex, st) != cudaSuccess) return cuda_fail(h, cudaGetLastError(), "cudaGraphLaunch");
  return KM_OK;
}

extern "C" {

int km_partition_sizes(int64_t n, int level_kind, int64_t level, int64_t* out_levels,
                       int64_t* out_nleaf, int64_t* out_nnonleaf) {
  Tree t;
  std::string msg;
  if (!build_tree(n, level_kind, level, &t, &msg)) return KM_ERR_BAD_ARG;
  if (out_levels) *out_levels = t.L;
  if (out_nleaf) *out_nleaf = t.nleaf;
  if (out_nnonleaf) *out_nnonleaf = t.nnode;
  return KM_OK;
}

int km_partition(int64_t n, int level_kind, int64_t level, int64_t* out_levels, int64_t* leaf,
                 int64_t* nonleaf) {
  Tree t;
  std::string msg;
  if (!build_tree(n, level_kind, level, &t, &msg)) return KM_ERR_BAD_ARG;
  if (out_levels) *out_levels = t.L;
  if (leaf) {
    for (int64_t j = 0; j < t.nleaf; ++j) {
      const int64_t s = t.leaf_start(j) + 1, e = s + t.leaf_size(j) - 1;
      leaf[4 * j] = s;
      leaf[4 * j + 1] = e;
      leaf[4 * j + 2] = s;
      leaf[4 * j + 3] = e;
    }
  }
  if (nonleaf) {
    // _nextlevel (indices.jl:40-51): rows = second child, cols = first child
    int64_t q = 0;
    for (int l = 1; l <= t.L; ++l) {
      for (int64_t k = 0; k < t.nodes_at(l); ++k) {
        const int64_t c1s = t.node_start(l - 1, 2 * k), c1n = t.node_size(l - 1, 2 * k);
        const int64_t c2s = t.node_start(l - 1, 2 * k + 1), c2n = t.node_size(l - 1, 2 * k + 1);
        nonleaf[4 * q] = c2s + 1;
        nonleaf[4 * q + 1] = c2s + c2n;
        nonleaf[4 * q + 2] = c1s + 1;
        nonleaf[4 * q + 3] = c1s + c1n;
        ++q;
      }
    }
  }
  return KM_OK;
}

int km_nystrom_landmarks(int64_t n, int64_t rank, int64_t* out) {
  if (n < 1 || rank < 2 || !out) return KM_ERR_BAD_ARG;
  // LinRange(1, n, rank)[i] = (1 - t) * 1 + t * n, t = (i-1)/(rank-1); round ties to even.
  for (int64_t i = 0; i < rank; ++i) {
    const double t = (double)i / (double)(rank - 1);
    const volatile double a = (1.0 - t) * 1.0;
    const volatile double b = t * (double)n;
    const double v = a + b;
    out[i] = (int64_t)std::nearbyint(v);
  }
  return KM_OK;
}

int km_create(const km_config* cfg, km_handle** out) {
  if (!out) return KM_ERR_BAD_ARG;
  *out = nullptr;
  km_handle* h = new km_handle();
  if (cfg) h->cfg = *cfg;
  if (h->cfg.precision != KM_PREC_FP64 && h->cfg.precision != KM_PREC_MIXED) {
    delete h;
    return KM_ERR_BAD_ARG;
  }
  h->mixed = (h->cfg.precision == KM_PREC_MIXED);
  if (h->cfg.refine_max_iter < 0) h->cfg.refine_max_iter = 0;
  if (h->cfg.refine_tol <= 0) h->cfg.refine_tol = 1e-10;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    delete h;
    return KM_ERR_CUDA;
  }
  if (h->cfg.device < 0 || h->cfg.device >= ndev) {
    delete h;
    return KM_ERR_BAD_ARG;
  }
  // The main stream runs at the highest priority and the side stream (solve operators formed
  // while the node levels run) at the lowest: a node-level CTA needs a whole SM, and when a level
  // ends the next level and the previous level's side work become ready together; the priorities
  // let the block scheduler place the critical-path CTAs first.
  int prio_low = 0, prio_high = 0;
  if (cudaSetDevice(h->cfg.device) != cudaSuccess ||
      cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high) != cudaSuccess ||
      cudaStreamCreateWithPriority(&h->stream, cudaStreamNonBlocking, prio_high) != cudaSuccess ||
      cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return KM_ERR_CUDA;
  }
  h->own_stream = h->stream;
  if (cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, prio_low) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return KM_ERR_CUDA;
  }
  for (auto& e : h->sev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  if (cudaStreamCreateWithPriority(&h->aux, cudaStreamNonBlocking, prio_low) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return KM_ERR_CUDA;
  }
  for (auto& e : h->xev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  for (auto& e : h->fev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  *out = h;
  return KM_OK;
}

int km_set_stream(km_handle* h, void* stream) {
  if (!h) return KM_ERR_BAD_ARG;
  cudaSetDevice(h->cfg.device);
  cudaStreamSynchronize(h->stream);
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return KM_OK;
}

int km_set_wait_limit(km_handle* h, int64_t polls) {
  if (!h) return KM_ERR_BAD_ARG;
  h->wait_limit = polls < 0 ? -1 : polls;
  h->alloc_epoch += 1;  // launch graphs captured with the previous limit are not replayed
  return KM_OK;
}

int km_profile_enable(km_handle* h, int on) {
  if (!h) return KM_ERR_BAD_ARG;
  cudaStreamSynchronize(h->stream);
  prof_resolve(h);
  h->prof = on != 0;
  for (int c = 0; c < KM_PROF_COUNT; ++c) {
    h->prof_ms[c] = 0.0;
    h->prof_n[c] = 0;
  }
  return KM_OK;
}

int km_profile_get(km_handle* h, int cls, double* total_ms, int64_t* launches) {
  if (!h || cls < 0 || cls >= KM_PROF_COUNT) return KM_ERR_BAD_ARG;
  cudaStreamSynchronize(h->stream);
  prof_resolve(h);
  if (total_ms) *total_ms = h->prof_ms[cls];
  if (launches) *launches = h->prof_n[cls];
  return KM_OK;
}

int km_destroy(km_handle* h) {
  if (!h) return KM_OK;
  cudaSetDevice(h->cfg.device);
  free_problem(h);
  if (h->fgraph) cudaGraphExecDestroy(h->fgraph);
  if (h->sgraph) cudaGraphExecDestroy(h->sgraph);
  prof_resolve(h);
  for (auto e : h->pool) cudaEventDestroy(e);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->side) cudaStreamSynchronize(h->side);
  for (auto e : h->sev)
    if (e) cudaEventDestroy(e);
  if (h->side) cudaStreamDestroy(h->side);
  if (h->aux) cudaStreamSynchronize(h->aux);
  for (auto e : h->xev)
    if (e) cudaEventDestroy(e);
  for (auto e : h->fev)
    if (e) cudaEventDestroy(e);
  if (h->aux) cudaStreamDestroy(h->aux);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  if (h->h_info) cudaFreeHost(h->h_info);
  delete h;
  return KM_OK;
}

const char* km_last_error(const km_handle* h) { return h ? h->err.c_str() : "null handle"; }

int km_get_stats(const km_handle* h, km_stats* out) {
  if (!h || !out) return KM_ERR_BAD_ARG;
  *out = h->stats;
  out->device_bytes = h->bytes;
  return KM_OK;
}


// ---- ACA assembly (src/HODLR/src/constructor.jl:44-53 with ACA, src/factorizations.jl:9-84) ----
static int aca_assemble(km_handle* h, const double* pts, bool dev, const Tree& t, const double* params,
                        int kernel_id, double tol, int64_t maxrank) {
  free_problem(h);
  h->tree = t;
  h->kp = make_kparams(kernel_id, params[0], params[1], params[2]);
  h->method = KM_METHOD_ACA;
  h->tol = tol;
  h->maxrank = maxrank;
  h->r = 0;
  cudaStream_t st = h->stream;
  // blocks, level 1 first (the reference's order of U[l][k], V[l][k])
  h->lvoff.assign(t.L + 2, 0);
  int64_t full = 0;
  for (int l = 1; l <= t.L; ++l) {
    h->lvoff[l] = (int64_t)h->blk.size();
    for (int64_t k = 0; k < t.nodes_at(l); ++k) {
      AcaBlock b{};
      b.col0 = t.node_start(l - 1, 2 * k);
      b.ncl = t.node_size(l - 1, 2 * k);
      b.row0 = t.node_start(l - 1, 2 * k + 1);
      b.nro = t.node_size(l - 1, 2 * k + 1);
      const int64_t minsz = std::min(b.nro, b.ncl);
      b.maxsz = (int)(maxrank == 0 ? minsz : std::min<int64_t>(maxrank, minsz));
      b.grid = minsz >= kAcaGridMin ? 1 : 0;
      full += (b.nro + b.ncl) * (int64_t)b.maxsz;
      h->blk.push_back(b);
    }
  }
  h->lvoff[t.L + 1] = (int64_t)h->blk.size();
  const int nb = (int)h->blk.size();
  // panel capacity: the largest column count (256 .. kAcaMaxCap, powers of two) whose panels
  // fit in 40% of the budget; the ACA kernel keeps two capacity-long vectors in shared memory
  int capmax = 256;
  for (int c = kAcaMaxCap; c > 256; c >>= 1) {
    int64_t tot = 0;
    for (const auto& b : h->blk) tot += (b.nro + b.ncl) * (int64_t)std::min(b.maxsz, c);
    if ((double)tot * 8.0 <= 0.4 * (double)device_budget(h)) {
      capmax = c;
      break;
    }
  }
  (void)full;
  int64_t offP = 0, offF = 0, offV = 0;
  int maxcap = 0;
  for (auto& b : h->blk) {
    b.cap = std::min(b.maxsz, capmax);
    b.offU = offP;
    offP += b.nro * b.cap;
    b.offV = offP;
    offP += b.ncl * b.cap;
    b.offFlag = offF;
    offF += b.nro + b.ncl;
    b.offPiv = offV;
    offV += b.cap;
    maxcap = std::max(maxcap, b.cap);
  }
  int64_t kbytes = 0;
  for (int64_t j = 0; j < t.nleaf; ++j) kbytes += t.leaf_size(j) * t.leaf_size(j);
  int rc;
  if ((rc = dalloc(h, &h->d_pts, 2 * t.n)) || (rc = dalloc(h, &h->d_K, kbytes)) || (rc = dalloc(h, &h->d_Lf, kbytes)) ||
      (rc = dalloc(h, &h->d_panels, offP)) || (rc = dalloc(h, &h->d_flags, offF)) ||
      (rc = dalloc(h, &h->d_piv, 2 * offV)) || (rc = dalloc(h, &h->d_brank, nb)) ||
      (rc = dalloc(h, &h->d_bstatus, nb)) || (rc = dalloc(h, &h->d_blk, nb)) ||
      (rc = dalloc(h, &h->d_info, t.nleaf + nb + 1)) || (rc = dalloc(h, &h->d_partial, kLogdetBlocks)) ||
      (rc = dalloc(h, &h->d_scalar, 4)) || (rc = dalloc(h, &h->d_gpartial, nb)) ||
      (rc = dalloc(h, &h->d_gsolve, nb)) || (rc = dalloc(h, &h->d_gnodes, nb))) {
    free_problem(h);
    return rc;
  }
  timer_start(h);
  KM_CUDA(h, cudaMemcpyAsync(h->d_pts, pts, sizeof(double) * 2 * t.n,
                             dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
  if (nb > 0) {
    KM_CUDA(h, cudaMemcpyAsync(h->d_blk, h->blk.data(), sizeof(AcaBlock) * nb, cudaMemcpyHostToDevice, st));
    KM_CUDA(h, cudaMemsetAsync(h->d_bstatus, 0, sizeof(int) * nb, st));
  }
  KLV(h, KM_PROF_EVAL, launch_eval_leaves(h->d_pts, t, h->kp, -1, h->d_K, st));
  if (nb > 0)
    KLV(h, KM_PROF_ACA, launch_aca(h->d_pts, h->kp, h->d_blk, nb, maxcap, h->d_panels, h->d_flags, h->d_piv, tol,
                                   h->d_brank, h->d_bstatus, st));
  // large blocks: one cooperative launch each, all SMs on one block
  {
    int gmax = 0;
    for (const auto& b : h->blk)
      if (b.grid) gmax = std::max(gmax, b.cap);
    if (gmax > 0) {
      if ((rc = grow(h, &h->d_acascr, aca_grid_scratch(gmax)))) return rc;
      for (int q = 0; q < nb; ++q) {
        if (!h->blk[q].grid) continue;
        bool ok = false;
        KLV(h, KM_PROF_ACA, ok = launch_aca_grid(h->d_pts, h->kp, h->d_blk, q, h->blk[q].cap, h->d_panels, h->d_flags,
                                                 h->d_piv, tol, h->d_brank, h->d_bstatus, h->d_acascr, st,
                                                 h->wait_limit));
        if (!ok)
          KLV(h, KM_PROF_ACA, launch_aca_one(h->d_pts, h->kp, h->d_blk, q, maxcap, h->d_panels, h->d_flags, h->d_piv,
                                             tol, h->d_brank, h->d_bstatus, st));
      }
    }
  }
  if ((rc = check_launch(h, "aca")) != KM_OK) return rc;
  h->stats.assemble_ms = timer_stop(h);
  if ((rc = sync(h, "aca")) != KM_OK) return rc;
  h->brank.assign(nb, 0);
  std::vector<int> stat(nb, 0);
  if (nb > 0) {
    KM_CUDA(h, cudaMemcpy(h->brank.data(), h->d_brank, sizeof(int) * nb, cudaMemcpyDeviceToHost));
    KM_CUDA(h, cudaMemcpy(stat.data(), h->d_bstatus, sizeof(int) * nb, cudaMemcpyDeviceToHost));
  }
  for (int q = 0; q < nb; ++q) {
    if (stat[q] == 1) return fail(h, KM_ERR_ACA, "Incompatible maxrank or matrix dimensions.");
    if (stat[q] == 3) return fail(h, KM_ERR_TIMEOUT, "a bounded grid barrier of the ACA kernel ran out");
    if (stat[q] == 2)
      return fail(h, KM_ERR_UNSUPPORTED, "ACA rank reached the panel capacity (" + std::to_string(capmax) +
                                             " columns) before the tolerance; pass a maxrank");
  }
  // node descriptors (factor storage sized by the ranks) and the per-block solve items
  int64_t r2 = 0;
  h->gmaxr = 1;
  for (int q = 0; q < nb; ++q) {
    r2 += (int64_t)h->brank[q] * h->brank[q];
    h->gmaxr = std::max(h->gmaxr, h->brank[q]);
  }
  if ((rc = dalloc(h, &h->d_R12, 2 * r2)) || (rc = dalloc(h, &h->d_CL, 2 * r2))) return rc;
  std::vector<GNodeDesc> nodes(nb);
  std::vector<GApplyItem> items(nb);
  int64_t o = 0;
  for (int q = 0; q < nb; ++q) {
    const AcaBlock& b = h->blk[q];
    const int rq = h->brank[q];
    GNodeDesc& N = nodes[q];
    N.Q1 = h->d_panels + b.offV;
    N.Q2 = h->d_panels + b.offU;
    N.R1 = h->d_R12 + 2 * o;
    N.R2 = h->d_R12 + 2 * o + (int64_t)rq * rq;
    N.C = h->d_CL + 2 * o;
    N.L22 = h->d_CL + 2 * o + (int64_t)rq * rq;
    N.s1 = b.ncl;
    N.s2 = b.nro;
    N.r = rq;
    o += (int64_t)rq * rq;
    items[q] = GApplyItem{q, 0, b.col0, b.row0, 0, nullptr, (b.nro + b.ncl >= kGapplyBig) ? 1 : 0};
  }
  h->gnodes_h = nodes;
  h->gsolve_h = items;
  if (nb > 0) {
    KM_CUDA(h, cudaMemcpy(h->d_gnodes, nodes.data(), sizeof(GNodeDesc) * nb, cudaMemcpyHostToDevice));
    KM_CUDA(h, cudaMemcpy(h->d_gsolve, items.data(), sizeof(GApplyItem) * nb, cudaMemcpyHostToDevice));
  }
  h->assembled = true;
  h->factorized = false;
  return KM_OK;
}

// ---- general factorisation (src/HODLR/src/symfact.jl:6-49) ----------------------------------
static int general_factorize(km_handle* h) {
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  const int nb = (int)h->blk.size();
  int rc;
  timer_start(h);
  KM_CUDA(h, cudaMemsetAsync(h->d_info, 0, sizeof(int) * (t.nleaf + nb + 1), st));  // + grid-barrier word
  if (!KL(h, KM_PROF_LEAF_CHOL, launch_leaf_chol<double>(h->d_K, h->d_Lf, t, h->d_info, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the leaf Cholesky kernel");
  if (nb > 0) {
    // leaf triangular solves of every panel (invapply!, src/HODLR/src/utils.jl:54-65)
    std::vector<LeafDesc> ld;
    for (int l = 1; l <= t.L; ++l) {
      for (int64_t k = 0; k < t.nodes_at(l); ++k) {
        const int q = (int)(h->lvoff[l] + k);
        const AcaBlock& b = h->blk[q];
        const int64_t j0 = k << l, jm = j0 + (int64_t(1) << (l - 1)), j1 = (k + 1) << l;
        for (int64_t j = j0; j < jm; ++j)
          ld.push_back(LeafDesc{j, h->d_panels + b.offV + (t.leaf_start(j) - b.col0), b.ncl, h->brank[q]});
        for (int64_t j = jm; j < j1; ++j)
          ld.push_back(LeafDesc{j, h->d_panels + b.offU + (t.leaf_start(j) - b.row0), b.nro, h->brank[q]});
      }
    }
    // per-level panel QR descriptors and W_l^{-1} updates of the coarser panels
    std::vector<PanelDesc> pd;
    std::vector<GApplyItem> fi;
    h->gfoff.assign(t.L + 2, 0);
    std::vector<int64_t> pdoff(t.L + 2, 0);
    int maxcols = 1;
    for (int l = 1; l <= t.L; ++l) {
      pdoff[l] = (int64_t)pd.size();
      h->gfoff[l] = (int64_t)fi.size();
      for (int64_t k = 0; k < t.nodes_at(l); ++k) {
        const int q = (int)(h->lvoff[l] + k);
        const AcaBlock& b = h->blk[q];
        int64_t o = 0;
        for (int p = 0; p < q; ++p) o += (int64_t)h->brank[p] * h->brank[p];
        const int rq = h->brank[q];
        pd.push_back(PanelDesc{h->d_panels + b.offV, b.ncl, b.ncl, rq, h->d_R12 + 2 * o, b.ncl >= kPanelBig ? 1 : 0});
        pd.push_back(PanelDesc{h->d_panels + b.offU, b.nro, b.nro, rq, h->d_R12 + 2 * o + (int64_t)rq * rq,
                               b.nro >= kPanelBig ? 1 : 0});
        for (int lev = l + 1; lev <= t.L; ++lev) {
          const int64_t kp = k >> (lev - l);
          const int qp = (int)(h->lvoff[lev] + kp);
          const AcaBlock& bp = h->blk[qp];
          const bool first = ((k >> (lev - l - 1)) & 1) == 0;  // node inside the ancestor's c1 side
          double* panel = h->d_panels + (first ? bp.offV : bp.offU);
          const int64_t side0 = first ? bp.col0 : bp.row0;
          const int64_t ldp = first ? bp.ncl : bp.nro;
          fi.push_back(GApplyItem{q, h->brank[qp], b.col0 - side0, b.row0 - side0, ldp, panel,
                                  (b.nro + b.ncl >= kGapplyBig) ? 1 : 0});
          maxcols = std::max(maxcols, h->brank[qp]);
        }
      }
    }
    pdoff[t.L + 1] = (int64_t)pd.size();
    h->gfoff[t.L + 1] = (int64_t)fi.size();
    dfree(h, h->d_ldesc);
    dfree(h, h->d_pdesc);
    dfree(h, h->d_gfact);
    h->d_ldesc = nullptr;
    h->d_pdesc = nullptr;
    h->d_gfact = nullptr;
    if ((rc = dalloc(h, &h->d_ldesc, (int64_t)ld.size())) || (rc = dalloc(h, &h->d_pdesc, (int64_t)pd.size())) ||
        (rc = dalloc(h, &h->d_gfact, std::max<int64_t>((int64_t)fi.size(), 1))))
      return rc;
    KM_CUDA(h, cudaMemcpy(h->d_ldesc, ld.data(), sizeof(LeafDesc) * ld.size(), cudaMemcpyHostToDevice));
    KM_CUDA(h, cudaMemcpy(h->d_pdesc, pd.data(), sizeof(PanelDesc) * pd.size(), cudaMemcpyHostToDevice));
    if (!fi.empty())
      KM_CUDA(h, cudaMemcpy(h->d_gfact, fi.data(), sizeof(GApplyItem) * fi.size(), cudaMemcpyHostToDevice));
    h->gfact_h = fi;
    // panel QR scratch (taus and block T factors) for the largest level
    std::vector<int> kmax_l(t.L + 2, 0);
    int64_t pqs = 1;
    for (int l = 1; l <= t.L; ++l) {
      for (int64_t p = pdoff[l]; p < pdoff[l + 1]; ++p) kmax_l[l] = std::max(kmax_l[l], pd[p].k);
      pqs = std::max(pqs, panel_qr_scratch((int)(pdoff[l + 1] - pdoff[l]), kmax_l[l]));
    }
    if ((rc = grow(h, &h->d_pqs, pqs))) return rc;
    if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri_desc(h->d_Lf, t, 0, h->d_ldesc, (int)ld.size(), h->gmaxr, st)))
      return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular solve kernel");
    for (int l = 1; l <= t.L; ++l) {
      const int np = (int)(pdoff[l + 1] - pdoff[l]);
      bool anybig = false;
      for (int64_t p = pdoff[l]; p < pdoff[l + 1]; ++p) anybig |= pd[p].big != 0;
      if (anybig) {
        if ((rc = grow(h, &h->d_pqg, panel_qr_gemm_scratch(pd.data() + pdoff[l], np, kmax_l[l])))) return rc;
        KLV(h, KM_PROF_LEAF_QR, launch_panel_qr_gemm(h->d_pdesc + pdoff[l], pd.data() + pdoff[l], np, kmax_l[l],
                                                     h->d_pqs, h->d_pqs + (int64_t)np * kmax_l[l], h->d_pqg,
                                                     h->d_info + t.nleaf + nb, st, h->wait_limit));
      } else {
        KLV(h, KM_PROF_LEAF_QR, launch_panel_qr(h->d_pdesc + pdoff[l], np, kmax_l[l], h->d_pqs,
                                                h->d_pqs + (int64_t)np * kmax_l[l], st));
      }
      KLV(h, KM_PROF_NODE, launch_gnode(h->d_gnodes + h->lvoff[l], (int)(h->lvoff[l + 1] - h->lvoff[l]),
                                        h->d_info + t.nleaf + h->lvoff[l], st));
      const int64_t a = h->gfoff[l], b = h->gfoff[l + 1];
      if (b > a && (rc = run_gapply(h, h->gfact_h, h->d_gfact, a, b, maxcols, 0, nullptr, nullptr, 0, 0)) != KM_OK)
        return rc;
    }
  }
  if ((rc = check_launch(h, "general factorize")) != KM_OK) return rc;
  h->stats.factorize_ms = timer_stop(h);
  if ((rc = sync(h, "general factorize")) != KM_OK) return rc;
  if ((rc = check_info(h, t.nleaf, "leaf")) != KM_OK) return rc;
  std::vector<int> info(nb + 1);
  KM_CUDA(h, cudaMemcpy(info.data(), h->d_info + t.nleaf, sizeof(int) * (nb + 1), cudaMemcpyDeviceToHost));
  if (info[nb]) return fail(h, KM_ERR_TIMEOUT, "a bounded grid barrier of the panel QR ran out");
  for (int q = 0; q < nb; ++q)
    if (info[q]) return fail(h, KM_ERR_NOT_SPD, "PosDefException: a low-rank capacitance block is not positive definite");
  h->factorized = true;
  return KM_OK;
}

static int assemble_impl(km_handle* h, const double* pts, bool dev, int64_t n, int kernel_id,
                         const double* params, int nparams, int method, double tol, int64_t maxrank,
                         int level_kind, int64_t level) {
  if (!h) return KM_ERR_BAD_ARG;
  cudaSetDevice(h->cfg.device);
  if (!pts || !params) return fail(h, KM_ERR_BAD_ARG, "null pointer");
  if (kernel_id != KM_KERNEL_RATQUAD && kernel_id != KM_KERNEL_MATERN32)
    return fail(h, KM_ERR_BAD_ARG, "unknown kernel id");
  if (nparams != 3 || !finite3(params)) return fail(h, KM_ERR_BAD_ARG, "need 3 finite parameters");
  if (!(params[1] > 0.0)) return fail(h, KM_ERR_BAD_ARG, "range parameter must be positive");
  if (method != KM_METHOD_NYSTROM && method != KM_METHOD_ACA)
    return fail(h, KM_ERR_BAD_ARG, "unknown method");
  Tree t;
  std::string msg;
  if (!build_tree(n, level_kind, level, &t, &msg)) return fail(h, KM_ERR_BAD_ARG, msg);
  if (t.nleaf > 65535) return fail(h, KM_ERR_UNSUPPORTED, "more than 65535 leaves");
  if (method == KM_METHOD_ACA) {
    if (!(tol >= 0.0) || maxrank < 0) return fail(h, KM_ERR_BAD_ARG, "ACA needs tol >= 0 and maxrank >= 0");
    h->leaf_tc = h->lf_holds_k = h->q_holds_phi = false;
    return aca_assemble(h, pts, dev, t, params, kernel_id, tol, maxrank);
  }
  // Nystrom checks (src/HODLR/src/constructor.jl:26-28)
  if (maxrank < 2) return fail(h, KM_ERR_BAD_ARG, "Please supply a fixed off-diagonal rank that is >=2.");
  const int64_t minleaf = t.m0;  // smallest leaf size
  if (maxrank >= minleaf - 1)
    return fail(h, KM_ERR_BAD_ARG, "Your nystrom rank is too big. Reduce the HODLR level or nystrom rank.");
  if (maxrank > kMaxNysRank) return fail(h, KM_ERR_UNSUPPORTED, "Nystrom rank above 80 is not supported");
  // Buffers are kept when the problem shape (n, levels, rank) is unchanged, so that repeated
  // assemblies (likelihood evaluations at new parameters) allocate nothing.
  // A new shape keeps every allocation that is large enough (grow); only a handle that last
  // held an ACA problem starts from scratch.
  if (h->d_blk) free_problem(h);
  const bool reuse = h->d_pts && h->tree.n == t.n && h->tree.L == t.L && h->r == (int)maxrank;
  if (!reuse) {
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->vcap = h->xcap = h->gcap = h->tcap = h->rcap = h->hcap = 0;
  }
  h->tree = t;
  h->kp = make_kparams(kernel_id, params[0], params[1], params[2]);
  h->method = method;
  h->tol = tol;
  h->maxrank = maxrank;
  h->r = (int)maxrank;
  h->assembled = h->factorized = false;
  h->dk_param = -1;
  h->d2_pair = -1;
  h->mixed = (h->cfg.precision == KM_PREC_MIXED);
  const int r = h->r;
  int64_t kbytes = 0;
  for (int64_t j = 0; j < t.nleaf; ++j) kbytes += t.leaf_size(j) * t.leaf_size(j);
  int rc;
  if (!reuse &&
      ((rc = grow(h, &h->d_pts, 2 * n)) || (rc = grow(h, &h->d_lnd, 2 * r)) ||
       (rc = grow(h, &h->d_lndidx, r)) || (rc = grow(h, &h->d_K, kbytes)) ||
       (rc = grow(h, &h->d_Lf, kbytes)) || (rc = grow(h, &h->d_Phi, n * r)) ||
       (rc = grow(h, &h->d_Q, n * r)) || (rc = grow(h, &h->d_tauleaf, t.nleaf * r)) ||
       (rc = grow(h, &h->d_R, (t.nleaf + t.nnode) * r * r)) || (rc = grow(h, &h->d_S, r * r)) ||
       (rc = grow(h, &h->d_Sc, r * r)) || (rc = grow(h, &h->d_SinvT, r * r)) || (rc = grow(h, &h->d_SinvTf, r * r)) ||
       (rc = grow(h, &h->d_Ct, std::max<int64_t>(t.nnode, 1) * r * r)) ||
       (rc = grow(h, &h->d_L22, std::max<int64_t>(t.nnode, 1) * r * r)) ||
       (rc = grow(h, &h->d_Eref, std::max<int64_t>(t.nnode, 1) * r * r)) ||
       (rc = grow(h, &h->d_Etau, std::max<int64_t>(t.nnode, 1) * r)) ||
       (rc = grow(h, &h->d_L22i, std::max<int64_t>(t.nnode, 1) * r * r)) ||
       (rc = grow(h, &h->d_E, std::max<int64_t>(t.nnode, 1) * 2 * r * r)) ||
       (rc = grow(h, &h->d_NT, std::max<int64_t>(t.nnode, 1) * 5 * r * r)) ||
       (rc = grow(h, &h->d_info, t.nleaf + t.nnode + 1)) ||
       (rc = grow(h, &h->d_partial, kLogdetBlocks)) || (rc = grow(h, &h->d_scalar, 4)))) {
    free_problem(h);
    return rc;
  }
  h->leaf_tc = h->mixed && leaf_tc_enabled() && leaf_chol_tc_supported(t, r);
  if (h->leaf_tc && (rc = grow(h, &h->d_lcscr, (leaf_chol_tc_scratch_bytes(t, r) + 7) / 8)) != KM_OK) {
    free_problem(h);
    return rc;
  }
  timer_start(h);
  cudaStream_t st = h->stream;
  KM_CUDA(h, cudaMemcpyAsync(h->d_pts, pts, sizeof(double) * 2 * n,
                             dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
  std::vector<int64_t> idx(r);
  km_nystrom_landmarks(n, r, idx.data());
  for (auto& v : idx) v -= 1;
  KM_CUDA(h, cudaMemcpyAsync(h->d_lndidx, idx.data(), sizeof(int64_t) * r, cudaMemcpyHostToDevice, st));
  KM_CUDA(h, cudaMemsetAsync(h->d_info, 0, sizeof(int) * (t.nleaf + t.nnode + 1), st));
  KLV(h, KM_PROF_EVAL, launch_gather_points(h->d_pts, h->d_lndidx, r, h->d_lnd, st));
  if (h->mixed) {
    if ((rc = grow(h, &h->d_pts3, 8 * n)) || (rc = grow(h, &h->d_lnd3, 8 * r))) return rc;
    KLV(h, KM_PROF_EVAL, launch_split_points(h->d_pts, n, h->d_pts3, st));
    KLV(h, KM_PROF_EVAL, launch_split_points(h->d_lnd, r, h->d_lnd3, st));
  }
  // S = K(P, P), its Cholesky factor and Sc^{-T} are single-CTA chains: they run on the side
  // stream while the leaves and the landmark columns are evaluated on the main stream
  side_begin(h);
  launch_eval_dense(h->d_lnd, r, h->d_lnd, r, h->kp, -1, h->d_S, r, h->side);
  KM_CUDA(h, cudaMemcpyAsync(h->d_Sc, h->d_S, sizeof(double) * r * r, cudaMemcpyDeviceToDevice, h->side));
  if (!launch_chol_small(h->d_Sc, r, h->d_info + t.nleaf + t.nnode, h->side)) {
    side_end(h);
    return fail(h, KM_ERR_UNSUPPORTED, "rank too large for the landmark Cholesky");
  }
  launch_tri_inv_t(h->d_Sc, r, h->d_SinvT, h->side);
  launch_to_ff(h->d_SinvT, P<ff>(h->d_SinvTf), (int64_t)r * r, h->side);
  h->stats.kernel_launches += 4;
  KLV(h, KM_PROF_EVAL, launch_eval_leaves(h->d_pts, t, h->kp, -1, h->d_K, st, h->mixed,
                                          h->leaf_tc ? P<ff>(h->d_Lf) : nullptr, h->mixed ? h->d_pts3 : nullptr));
  h->lf_holds_k = h->leaf_tc;
  KLV(h, KM_PROF_EVAL, launch_eval_phi(h->d_pts, h->d_lnd, r, t, h->kp, -1, h->d_Phi, st, h->mixed,
                                       h->mixed ? h->d_pts3 : nullptr, h->mixed ? h->d_lnd3 : nullptr,
                                       h->mixed ? P<ff>(h->d_Q) : nullptr));
  h->q_holds_phi = h->mixed;
  side_end(h);
  if ((rc = check_launch(h, "assemble")) != KM_OK) return rc;
  if ((rc = fetch_info_async(h, t.nleaf + t.nnode + 1)) != KM_OK) return rc;  // last word: chol(S) status
  h->stats.assemble_ms = timer_stop(h);
  if ((rc = sync(h, "assemble")) != KM_OK) return rc;
  if (h->h_info[t.nleaf + t.nnode] != 0)
    return fail(h, KM_ERR_NOT_SPD, "PosDefException: landmark matrix K(P, P) is not positive definite");
  h->assembled = true;
  h->factorized = false;
  return KM_OK;
}

int km_assemble(km_handle* h, const double* pts, int64_t n, int kernel_id, const double* params,
                int nparams, int method, double tol, int64_t maxrank, int level_kind,
                int64_t level) {
  return assemble_impl(h, pts, false, n, kernel_id, params, nparams, method, tol, maxrank,
                       level_kind, level);
}

int km_assemble_dev(km_handle* h, const double* d_pts, int64_t n, int kernel_id,
                    const double* params, int nparams, int method, double tol, int64_t maxrank,
                    int level_kind, int64_t level) {
  return assemble_impl(h, d_pts, true, n, kernel_id, params, nparams, method, tol, maxrank,
                       level_kind, level);
}

// The launch sequence of the nested Nystrom factorisation (main stream, side stream forked for
// the solve operators), without host synchronisation, so that it can be captured in a graph.
// Forward half of the solve, X <- W^{-1} X (nested_fwd_t), enqueued on the aux stream at the
// factorisation's dependency points: the leaf solve as soon as the leaf factor is final, the leaf
// projections once the explicit leaf bases exist, the up-sweep of level l once level l is
// finalised, the down-sweep and the expansion after the last level.  Same kernels and order as
// nested_fwd_t, so the same bits.
extern "C++" {
template <typename T>
static void aux_fwd_leaf(km_handle* h) {
  auto* job = h->fwd_job;
  const Tree& t = h->tree;
  cudaStream_t ax = h->aux;
  cudaEventRecord(h->xev[0], h->stream);
  cudaStreamWaitEvent(ax, h->xev[0], 0);
  T* X = reinterpret_cast<T*>(job->X);
  if constexpr (std::is_same<T, ff>::value) {
    launch_to_ff(job->X, X, t.n * job->k, ax);
    job->ok = use_tri_blk(h, job->k) ? launch_leaf_tri_blk(P<ff>(h->d_Lf), t, 0, X, t.n, job->k, ax)
                         : launch_leaf_tri<ff>(P<ff>(h->d_Lf), t, 0, X, 1, t.n, 0, X, 1, t.n, 0, job->k, ax);
  } else {
    job->ok = launch_leaf_tri<double>(h->d_Lf, t, 0, X, 1, t.n, 0, X, 1, t.n, 0, job->k, ax);
  }
  h->stats.kernel_launches += 2;
}

template <typename T>
static void aux_fwd_nodes(km_handle* h) {
  auto* job = h->fwd_job;
  const Tree& t = h->tree;
  cudaStream_t ax = h->aux;
  T* X = reinterpret_cast<T*>(job->X);
  const int k = job->k;
  if (t.L > 0) {
    NodeMatsH nm = node_mats(h);
    cudaStreamWaitEvent(ax, h->xev[1], 0);
    launch_leaf_proj<T>(P<T>(h->d_Q), P<T>(h->d_tauleaf), h->r, t, X, t.n, P<T>(h->d_VP), k, ax);
    for (int l = 1; l <= t.L; ++l) {
      cudaStreamWaitEvent(ax, h->fev[l], 0);
      launch_up<T>(t, nm, l, P<T>(h->d_VP), P<T>(h->d_VD), k, UP_FWD_, ax);
    }
    for (int l = t.L; l >= 1; --l)
      launch_down<T>(t, nm, l, P<T>(h->d_VP), P<T>(h->d_VG), P<T>(h->d_VD), k, DN_FWD_, ax);
    launch_leaf_expand<T>(P<T>(h->d_Q), P<T>(h->d_tauleaf), h->r, t, P<T>(h->d_VG), X, t.n, k, -1.0, ax);
    h->stats.kernel_launches += 2 + 2 * t.L;
  }
  cudaEventRecord(h->xev[2], ax);
  cudaStreamWaitEvent(h->stream, h->xev[2], 0);
}

}  // extern "C++"

static int factorize_launches(km_handle* h) {
  const Tree& t = h->tree;
  const int r = h->r;
  cudaStream_t st = h->stream;
  const bool fwd = h->fwd_job != nullptr;
  KM_CUDA(h, cudaMemsetAsync(h->d_info, 0, sizeof(int) * (t.nleaf + t.nnode), st));
  if (h->mixed && h->leaf_tc) {
    // L_j and A_j = L_j^{-1} Phi_j from one blocked Cholesky of [K_j; Phi_j'] whose trailing
    // updates run on the tensor cores (km_leaf_tc.cu)
    if (!h->q_holds_phi) KLV(h, KM_PROF_OTHER, launch_to_ff(h->d_Phi, P<ff>(h->d_Q), t.n * r, st));
    for (int p = 0; p < leaf_chol_tc_steps(t); ++p) {
      KLV(h, KM_PROF_LEAF_CHOL, launch_leaf_chol_tc_diag(P<ff>(h->d_Lf), r, t, p, h->d_lcscr, h->d_info, st));
      KLV(h, KM_PROF_LEAF_TC, launch_leaf_chol_tc_trsm(P<ff>(h->d_Lf), P<ff>(h->d_Q), r, t, p, h->d_lcscr,
                                                       h->d_info, st));
      if (leaf_chol_tc_has_update(t, p))
        KLV(h, KM_PROF_LEAF_TC, launch_leaf_chol_tc_update(P<ff>(h->d_Lf), P<ff>(h->d_Q), r, t, p, h->d_lcscr,
                                                           h->d_info, st));
    }
    if (fwd) aux_fwd_leaf<ff>(h);
  } else if (!(h->mixed ? KL(h, KM_PROF_LEAF_CHOL, launch_leaf_chol<ff>(h->d_K, P<ff>(h->d_Lf), t, h->d_info, st))
                        : KL(h, KM_PROF_LEAF_CHOL, launch_leaf_chol<double>(h->d_K, h->d_Lf, t, h->d_info, st)))) {
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the leaf Cholesky kernel");
  }
  // A = L^{-1} Phi on every leaf, then Householder QR of each leaf panel
  if (h->mixed) {
    // float-pair factor: every FP64-pipe-bound step runs on the FP32 pipe in float-float
    if (!h->leaf_tc) {
      if (!h->q_holds_phi) KLV(h, KM_PROF_OTHER, launch_to_ff(h->d_Phi, P<ff>(h->d_Q), t.n * r, st));
      if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri<ff>(P<ff>(h->d_Lf), t, 0, P<ff>(h->d_Q), r, 0, 1, P<ff>(h->d_Q),
                                                       r, 0, 1, r, st)))
        return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular solve kernel");
      if (fwd) aux_fwd_leaf<ff>(h);
    }
    if (t.L > 0) {
      KLV(h, KM_PROF_LEAF_QR, launch_leaf_qr<ff>(P<ff>(h->d_Q), r, t, P<ff>(h->d_tauleaf), P<ff>(h->d_R), st));
      side_begin(h);
      launch_leaf_formq<ff>(P<ff>(h->d_Q), P<ff>(h->d_tauleaf), r, t, h->side);
      if (fwd) cudaEventRecord(h->xev[1], h->side);
      for (int l = 1; l <= t.L; ++l) {
        KLV(h, KM_PROF_NODE, launch_node_factor<ff>(P<ff>(h->d_R), P<ff>(h->d_SinvTf), r, l, t, P<ff>(h->d_Ct),
                                                    P<ff>(h->d_L22), P<ff>(h->d_Eref), P<ff>(h->d_Etau),
                                                    h->d_info + t.nleaf, st, h->node_cluster_max,
                                                    (int)std::min<int64_t>(h->wait_limit, INT32_MAX)));
        side_level(h, l);
        {
          const NodeMatsH nm = node_mats(h);
          launch_node_finalize<ff>(P<ff>(h->d_L22), P<ff>(h->d_Ct), P<ff>(h->d_Eref), P<ff>(h->d_Etau), r, l, t,
                                   P<ff>(h->d_L22i), P<ff>(h->d_E), P<ff>((double*)nm.CtT), P<ff>((double*)nm.L22T),
                                   P<ff>((double*)nm.L22iT), P<ff>((double*)nm.ET), h->side);
        }
        if (fwd) cudaEventRecord(h->fev[l], h->side);
      }
      side_end(h);
    }
    if (fwd) aux_fwd_nodes<ff>(h);
  } else {
    KM_CUDA(h, cudaMemcpyAsync(h->d_Q, h->d_Phi, sizeof(double) * t.n * r, cudaMemcpyDeviceToDevice, st));
    if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri<double>(h->d_Lf, t, 0, h->d_Q, r, 0, 1, h->d_Q, r, 0, 1, r, st)))
      return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular solve kernel");
    if (fwd) aux_fwd_leaf<double>(h);
    if (t.L > 0) {
      KLV(h, KM_PROF_LEAF_QR, launch_leaf_qr<double>(h->d_Q, r, t, h->d_tauleaf, h->d_R, st));
      side_begin(h);
      launch_leaf_formq<double>(h->d_Q, h->d_tauleaf, r, t, h->side);
      if (fwd) cudaEventRecord(h->xev[1], h->side);
      for (int l = 1; l <= t.L; ++l) {
        KLV(h, KM_PROF_NODE, launch_node_factor<double>(h->d_R, h->d_SinvT, r, l, t, h->d_Ct, h->d_L22, h->d_Eref,
                                                        h->d_Etau, h->d_info + t.nleaf, st));
        side_level(h, l);
        {
          const NodeMatsH nm = node_mats(h);
          launch_node_finalize<double>(h->d_L22, h->d_Ct, h->d_Eref, h->d_Etau, r, l, t, h->d_L22i, h->d_E,
                                       (double*)nm.CtT, (double*)nm.L22T, (double*)nm.L22iT, (double*)nm.ET,
                                       h->side);
        }
        if (fwd) cudaEventRecord(h->fev[l], h->side);
      }
      side_end(h);
    }
    if (fwd) aux_fwd_nodes<double>(h);
  }
  return KM_OK;
}

int km_factorize(km_handle* h) {
  if (!h) return KM_ERR_BAD_ARG;
  cudaSetDevice(h->cfg.device);
  if (!h->assembled) return fail(h, KM_ERR_STATE, "assemble first");
  if (h->method == KM_METHOD_ACA) {
    if (h->factorized)
      return fail(h, KM_ERR_STATE, "already factorised (U and V were overwritten); assemble again");
    return general_factorize(h);
  }
  const Tree& t = h->tree;
  const int r = h->r;
  cudaStream_t st = h->stream;
  int rc;
  timer_start(h);
  if (h->mixed && h->leaf_tc && !h->lf_holds_k) {
    // a second factorisation of the same assembly: the leaf matrices evaluated again (the same
    // kernel on the same points, so the same float pairs and FP64 values as the assembly's)
    KLV(h, KM_PROF_EVAL, launch_eval_leaves(h->d_pts, t, h->kp, -1, h->d_K, st, true, P<ff>(h->d_Lf), h->d_pts3));
  }
  if (h->mixed && !h->q_holds_phi) {
    // likewise the float pairs of Phi (a conversion of the FP64 copy could pick the other of two
    // pairs with the same value, and the factor would differ in its last bits)
    KLV(h, KM_PROF_EVAL, launch_eval_phi(h->d_pts, h->d_lnd, r, t, h->kp, -1, h->d_Phi, st, true, h->d_pts3,
                                         h->d_lnd3, P<ff>(h->d_Q)));
    h->q_holds_phi = true;
  }
  h->lf_holds_k = false;
  const int64_t fk[6] = {(int64_t)h->alloc_epoch, t.n, t.L, r, h->mixed ? 1 : 0, h->q_holds_phi ? 1 : 0};
  auto* job = h->fwd_job;  // km_factorize_solve_dev: the forward half of a solve rides along
  if (job)
    rc = factorize_launches(h);
  else
    rc = run_graphed(h, &h->fgraph, h->fkey, fk, [&]() -> int { return factorize_launches(h); });
  h->q_holds_phi = false;  // the factorisation works on d_Q in place
  if (rc != KM_OK) return rc;
  if ((rc = check_launch(h, "factorize")) != KM_OK) return rc;
  if ((rc = fetch_info_async(h, t.nleaf + t.nnode)) != KM_OK) return rc;  // leaf and node pivot status
  h->stats.factorize_ms = timer_stop(h);
  if ((rc = sync(h, "factorize")) != KM_OK) return rc;
  rc = check_info_words(h, h->h_info, t.nleaf, "leaf");
  if (rc == KM_OK) {
    const int* info = h->h_info + t.nleaf;
    for (int64_t i = 0; i < t.nnode && rc == KM_OK; ++i) {
      if (info[i] < 0) return fail(h, KM_ERR_TIMEOUT, "a bounded wait inside the node factorisation ran out");
      if (info[i]) rc = fail(h, KM_ERR_NOT_SPD, "PosDefException: a low-rank capacitance block is not positive definite");
    }
  }
  if (rc == KM_ERR_NOT_SPD && h->mixed) {
    // A pivot that is positive in FP64 can round to <= 0 in float pairs when the capacitance
    // I - Ct'Ct is close to singular (smooth kernels, large range).  Redo this problem in FP64;
    // the next assembly returns to the configured precision.
    h->mixed = false;
    h->stats.precision_fallbacks += 1;
    if (job) {  // the forward half ran on the float-pair factor: the caller solves again
      job->ok = false;
      h->fwd_job = nullptr;
    }
    return km_factorize(h);
  }
  if (rc != KM_OK) return rc;
  h->factorized = true;
  return KM_OK;
}

int km_matvec_dev(km_handle* h, const double* d_x, double* d_y, int64_t k) {
  if (!h || !d_x || !d_y || k < 1) return fail(h, KM_ERR_BAD_ARG, "bad matvec arguments");
  cudaSetDevice(h->cfg.device);
  if (!h->assembled) return fail(h, KM_ERR_STATE, "assemble first");
  int rc;
  if ((rc = ensure_vec(h, k)) != KM_OK) return rc;
  timer_start(h);
  if (h->factorized) {
    // mul!(target, K, src) after factorisation: W (W' x)  (baseoverloads.jl:170-177)
    KM_CUDA(h, cudaMemcpyAsync(d_y, d_x, sizeof(double) * h->tree.n * k, cudaMemcpyDeviceToDevice, h->stream));
    if ((rc = nested_mul_t(h, d_y, (int)k)) != KM_OK) return rc;
    if ((rc = nested_mul(h, d_y, (int)k)) != KM_OK) return rc;
  } else {
    if ((rc = nystrom_matvec(h, d_x, d_y, (int)k)) != KM_OK) return rc;
  }
  h->stats.matvec_ms = timer_stop(h);
  return sync(h, "matvec");
}

// symmetricfactorize!(HK) followed by HK \ b (symfact.jl:6-49, baseoverloads.jl:181-192) in one
// call, as LAPACK's posv combines potrf and potrs: the forward half of the solve runs on the aux
// stream behind the factorisation's dependency points (aux_fwd_leaf, aux_fwd_nodes), using the
// SMs that the upper node levels leave idle; the backward half and the refinement follow as in
// km_solve_dev.  Same kernels in the same order as km_factorize + km_solve_dev, so the same
// results; ACA handles take those two calls.
int km_factorize_solve_dev(km_handle* h, const double* d_b, double* d_x, int64_t k) {
  if (!h || !d_b || !d_x || k < 1) return fail(h, KM_ERR_BAD_ARG, "bad solve arguments");
  cudaSetDevice(h->cfg.device);
  if (!h->assembled) return fail(h, KM_ERR_STATE, "assemble first");
  int rc;
  if (h->method != KM_METHOD_NYSTROM) {
    if ((rc = km_factorize(h)) != KM_OK) return rc;
    return km_solve_dev(h, d_b, d_x, k);
  }
  if ((rc = ensure_vec(h, k)) != KM_OK) return rc;
  const int64_t n = h->tree.n;
  const double* b_keep = d_b;
  if (d_x != d_b) {
    KM_CUDA(h, cudaMemcpyAsync(d_x, d_b, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, h->stream));
  } else {
    // in place: the right-hand sides are kept for the refinement, or for a second solve after a
    // precision fallback
    if ((rc = grow(h, &h->d_bkeep, n * k)) != KM_OK) return rc;
    KM_CUDA(h, cudaMemcpyAsync(h->d_bkeep, d_b, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, h->stream));
    b_keep = h->d_bkeep;
  }
  km_handle::FwdJob job{d_x, (int)k, true};
  h->fwd_job = &job;
  rc = km_factorize(h);
  h->fwd_job = nullptr;
  if (rc != KM_OK) return rc;
  if (!job.ok) return km_solve_dev(h, b_keep, d_x, k);
  timer_start(h);
  if (h->mixed) {
    ff* Xf = reinterpret_cast<ff*>(d_x);
    if ((rc = nested_bwd_t<ff>(h, Xf, (int)k, true)) != KM_OK) return rc;
    KLV(h, KM_PROF_OTHER, launch_from_ff(Xf, d_x, n * k, h->stream));
  } else if ((rc = nested_bwd_t<double>(h, d_x, (int)k, true)) != KM_OK) {
    return rc;
  }
  if (h->mixed && h->cfg.refine_max_iter > 0 && (rc = refine(h, b_keep, d_x, (int)k)) != KM_OK) return rc;
  h->stats.solve_ms = timer_stop(h);
  return sync(h, "solve");
}

int km_solve_dev(km_handle* h, const double* d_b, double* d_x, int64_t k) {
  if (!h || !d_b || !d_x || k < 1) return fail(h, KM_ERR_BAD_ARG, "bad solve arguments");
  cudaSetDevice(h->cfg.device);
  if (!h->factorized) return fail(h, KM_ERR_STATE, "No solves without factorization.");
  int rc;
  if ((rc = ensure_vec(h, k)) != KM_OK) return rc;
  const bool refining = h->mixed && h->method == KM_METHOD_NYSTROM && h->cfg.refine_max_iter > 0;
  if (refining && k > h->rcap) {
    h->rcap = 0;
    if ((rc = grow(h, &h->d_res, 2 * h->tree.n * k)) || (rc = grow(h, &h->d_rdots, 2 * k))) return rc;
    h->rcap = k;
  }
  timer_start(h);
  const double* b_keep = d_b;
  if (d_x != d_b) {
    KM_CUDA(h, cudaMemcpyAsync(d_x, d_b, sizeof(double) * h->tree.n * k, cudaMemcpyDeviceToDevice, h->stream));
  } else if (refining) {
    // in place: the refinement residual needs the right-hand sides after x has replaced them
    double* keep = h->d_res + h->tree.n * k;
    KM_CUDA(h, cudaMemcpyAsync(keep, d_b, sizeof(double) * h->tree.n * k, cudaMemcpyDeviceToDevice, h->stream));
    b_keep = keep;
  }
  if (h->method == KM_METHOD_NYSTROM) {
    const int64_t sk[7] = {(int64_t)h->alloc_epoch, h->tree.n, h->tree.L, h->r, h->mixed ? 1 : 0,
                           (int64_t)(uintptr_t)d_x, k};
    rc = run_graphed(h, &h->sgraph, h->skey, sk, [&]() -> int { return nested_solve(h, d_x, (int)k); });
  } else {
    rc = nested_solve(h, d_x, (int)k);
  }
  if (rc != KM_OK) return rc;
  if (refining && (rc = refine(h, b_keep, d_x, (int)k)) != KM_OK) return rc;
  h->stats.solve_ms = timer_stop(h);
  return sync(h, "solve");
}

int km_factor_solve_dev(km_handle* h, int transpose, const double* d_b, double* d_x, int64_t k) {
  if (!h || !d_b || !d_x || k < 1) return fail(h, KM_ERR_BAD_ARG, "bad solve arguments");
  cudaSetDevice(h->cfg.device);
  if (!h->factorized) return fail(h, KM_ERR_STATE, "factorize first");
  int rc;
  if ((rc = ensure_vec(h, k)) != KM_OK) return rc;
  if (d_x != d_b)
    KM_CUDA(h, cudaMemcpyAsync(d_x, d_b, sizeof(double) * h->tree.n * k, cudaMemcpyDeviceToDevice, h->stream));
  rc = transpose ? nested_bwd(h, d_x, (int)k) : nested_fwd(h, d_x, (int)k);
  if (rc != KM_OK) return rc;
  return sync(h, "factor_solve");
}

int km_factor_mul_dev(km_handle* h, int transpose, const double* d_b, double* d_x, int64_t k) {
  if (!h || !d_b || !d_x || k < 1) return fail(h, KM_ERR_BAD_ARG, "bad product arguments");
  cudaSetDevice(h->cfg.device);
  if (!h->factorized) return fail(h, KM_ERR_STATE, "factorize first");
  int rc;
  if ((rc = ensure_vec(h, k)) != KM_OK) return rc;
  if (d_x != d_b)
    KM_CUDA(h, cudaMemcpyAsync(d_x, d_b, sizeof(double) * h->tree.n * k, cudaMemcpyDeviceToDevice, h->stream));
  rc = transpose ? nested_mul_t(h, d_x, (int)k) : nested_mul(h, d_x, (int)k);
  if (rc != KM_OK) return rc;
  return sync(h, "factor_mul");
}

// host-pointer wrappers: copy in, run on the device, copy out
static int host_call(km_handle* h, const double* b, double* x, int64_t k,
                     int (*fn)(km_handle*, const double*, double*, int64_t)) {
  if (!h || !b || !x || k < 1) return fail(h, KM_ERR_BAD_ARG, "bad arguments");
  cudaSetDevice(h->cfg.device);
  if (!h->assembled) return fail(h, KM_ERR_STATE, "assemble first");
  int rc;
  if ((rc = ensure_xy(h, k)) != KM_OK) return rc;
  const size_t bytes = sizeof(double) * h->tree.n * k;
  KM_CUDA(h, cudaMemcpyAsync(h->d_X, b, bytes, cudaMemcpyHostToDevice, h->stream));
  if ((rc = fn(h, h->d_X, h->d_Y, k)) != KM_OK) return rc;
  KM_CUDA(h, cudaMemcpyAsync(x, h->d_Y, bytes, cudaMemcpyDeviceToHost, h->stream));
  return sync(h, "copy out");
}

int km_matvec(km_handle* h, const double* x, double* y, int64_t k) { return host_call(h, x, y, k, km_matvec_dev); }
int km_factorize_solve(km_handle* h, const double* b, double* x, int64_t k) {
  return host_call(h, b, x, k, km_factorize_solve_dev);
}
int km_solve(km_handle* h, const double* b, double* x, int64_t k) { return host_call(h, b, x, k, km_solve_dev); }

static int fs0(km_handle* h, const double* b, double* x, int64_t k) { return km_factor_solve_dev(h, 0, b, x, k); }
static int fs1(km_handle* h, const double* b, double* x, int64_t k) { return km_factor_solve_dev(h, 1, b, x, k); }
static int fm0(km_handle* h, const double* b, double* x, int64_t k) { return km_factor_mul_dev(h, 0, b, x, k); }
static int fm1(km_handle* h, const double* b, double* x, int64_t k) { return km_factor_mul_dev(h, 1, b, x, k); }

int km_factor_solve(km_handle* h, int transpose, const double* b, double* x, int64_t k) {
  return host_call(h, b, x, k, transpose ? fs1 : fs0);
}
int km_factor_mul(km_handle* h, int transpose, const double* b, double* x, int64_t k) {
  return host_call(h, b, x, k, transpose ? fm1 : fm0);
}

int km_logdet(km_handle* h, double* out) {
  if (!h || !out) return fail(h, KM_ERR_BAD_ARG, "bad logdet arguments");
  cudaSetDevice(h->cfg.device);
  if (!h->factorized) return fail(h, KM_ERR_STATE, "No logdet without factorization.");
  timer_start(h);
  int rc;
  if (h->method == KM_METHOD_ACA) {
    // 2 sum log diag(L_leaf) + 2 sum log|diag(L22)| (baseoverloads.jl:194-209), summed on the host
    // in a fixed order
    Tree t0 = h->tree;
    t0.nnode = 0;
    const int nb = (int)h->blk.size();
    KLV(h, KM_PROF_OTHER, launch_logdet<double>(h->d_Lf, t0, nullptr, 1, h->d_partial, kLogdetBlocks, h->d_scalar,
                                                h->stream));
    if (nb > 0) KLV(h, KM_PROF_OTHER, launch_glogdet(h->d_gnodes, nb, h->d_gpartial, h->stream));
    if ((rc = check_launch(h, "logdet")) != KM_OK) return rc;
    double leaf = 0.0;
    std::vector<double> part(nb);
    KM_CUDA(h, cudaMemcpyAsync(&leaf, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (nb > 0) KM_CUDA(h, cudaMemcpyAsync(part.data(), h->d_gpartial, sizeof(double) * nb, cudaMemcpyDeviceToHost, h->stream));
    if ((rc = sync(h, "logdet")) != KM_OK) return rc;
    double s = leaf;
    for (int q = 0; q < nb; ++q) s += part[q];
    *out = s;
    h->stats.logdet_ms = timer_stop(h);
    return KM_OK;
  }
  if (h->mixed)
    KLV(h, KM_PROF_OTHER, launch_logdet<ff>(P<ff>(h->d_Lf), h->tree, P<ff>(h->d_L22), h->r, h->d_partial,
                                            kLogdetBlocks, h->d_scalar, h->stream));
  else
    KLV(h, KM_PROF_OTHER, launch_logdet<double>(h->d_Lf, h->tree, h->d_L22, h->r, h->d_partial, kLogdetBlocks,
                                                h->d_scalar, h->stream));
  h->stats.kernel_launches += 1;  // the logdet runs a partial and a final reduction kernel
  if ((rc = check_launch(h, "logdet")) != KM_OK) return rc;
  // the end mark goes before the read-back, so the one synchronisation below covers both
  cudaEventRecord(h->ev1, h->stream);
  KM_CUDA(h, cudaMemcpyAsync(out, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if ((rc = sync(h, "logdet")) != KM_OK) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  h->stats.logdet_ms = ms;
  return KM_OK;
}

int km_block_ranks(km_handle* h, int64_t* out) {
  if (!h || !out) return fail(h, KM_ERR_BAD_ARG, "null");
  if (!h->assembled) return fail(h, KM_ERR_STATE, "assemble first");
  for (int64_t q = 0; q < h->tree.nnode; ++q)
    out[q] = (h->method == KM_METHOD_ACA) ? h->brank[q] : h->r;
  return KM_OK;
}

int km_aca_pivots(km_handle* h, int64_t block, int64_t cap, int64_t* rows, int64_t* cols, int64_t* out_rank) {
  if (!h || !rows || !cols || !out_rank) return fail(h, KM_ERR_BAD_ARG, "null");
  if (!h->assembled || h->method != KM_METHOD_ACA) return fail(h, KM_ERR_STATE, "no ACA assembly");
  if (block < 0 || block >= (int64_t)h->blk.size()) return fail(h, KM_ERR_BAD_ARG, "block out of range");
  const AcaBlock& b = h->blk[block];
  const int rq = h->brank[block];
  std::vector<int> p(2 * (size_t)b.cap);
  KM_CUDA(h, cudaMemcpy(p.data(), h->d_piv + 2 * b.offPiv, sizeof(int) * 2 * b.cap, cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < std::min<int64_t>(cap, rq); ++i) {
    rows[i] = p[i];
    cols[i] = p[b.cap + i];
  }
  *out_rank = rq;
  return KM_OK;
}

int km_block_factors(km_handle* h, int64_t block, double* U, double* V) {
  if (!h || !U || !V) return fail(h, KM_ERR_BAD_ARG, "null");
  if (!h->assembled || h->method != KM_METHOD_ACA) return fail(h, KM_ERR_STATE, "no ACA assembly");
  if (h->factorized) return fail(h, KM_ERR_STATE, "U and V abandoned after overwriting");
  if (block < 0 || block >= (int64_t)h->blk.size()) return fail(h, KM_ERR_BAD_ARG, "block out of range");
  const AcaBlock& b = h->blk[block];
  const int rq = h->brank[block];
  KM_CUDA(h, cudaMemcpy(U, h->d_panels + b.offU, sizeof(double) * b.nro * rq, cudaMemcpyDeviceToHost));
  KM_CUDA(h, cudaMemcpy(V, h->d_panels + b.offV, sizeof(double) * b.ncl * rq, cudaMemcpyDeviceToHost));
  return KM_OK;
}

int km_derivative_matvec(km_handle* h, int param, const double* x, double* y, int64_t k) {
  if (!h || !x || !y || k < 1 || param < 0 || param > 2) return fail(h, KM_ERR_BAD_ARG, "bad derivative arguments");
  cudaSetDevice(h->cfg.device);
  if (!h->assembled) return fail(h, KM_ERR_STATE, "assemble first");
  if (h->method != KM_METHOD_NYSTROM) return fail(h, KM_ERR_STATE, "This is only valid for Nystrom-block matrices.");
  int rc;
  if ((rc = ensure_xy(h, k)) != KM_OK) return rc;
  const size_t bytes = sizeof(double) * h->tree.n * k;
  KM_CUDA(h, cudaMemcpyAsync(h->d_X, x, bytes, cudaMemcpyHostToDevice, h->stream));
  if ((rc = derivative_apply(h, param, h->d_X, h->d_Y, (int)k)) != KM_OK) return rc;
  KM_CUDA(h, cudaMemcpyAsync(y, h->d_Y, bytes, cudaMemcpyDeviceToHost, h->stream));
  return sync(h, "derivative_matvec");
}

// negloglik (maxlikfunctions.jl:2-9) and stoch_gradient (stochasticgradient.jl:30-44):
//   alpha = K^{-1} y,  nll = 0.5 logdet K + 0.5 y' alpha,
//   T = W'^{-1} V (one factor solve for all probes, shared by the three parameters),
//   g_j = 0.5 (mean_v t_v' dK_j t_v - alpha' dK_j alpha).
// The data term y' K^{-1} dK_j K^{-1} y of HODLR_grad_term (stochasticgradient.jl:22-25) is
// evaluated as alpha' dK_j alpha, which is the same quantity since K^{-1} is symmetric.
// With `profile` the scale is profiled out (profile_negloglik, maxlikfunctions.jl:11-19;
// HODLR_p_grad_term, stochasticgradient.jl:48-64): nll = 0.5 (logdet K + n log(y' alpha)) and
// g_j = 0.5 (mean_v t_v' dK_j t_v - n alpha' dK_j alpha / y' alpha), from the same solves.
// With `fisher` the stochastic Fisher matrix of stoch_fisher (stochastichessian.jl:91-115) and
// grad_and_fisher_matrix (:152-181) is formed from the same probes: A_j = W^{-1} dK_j T,
// F_jk = 0.5 mean_v (A_j v)'(A_k v).  The reference forms the off-diagonal entries by
// polarisation, 0.5 (0.5 mean |A_j v + A_k v|^2 - F_jj - F_kk), which is the same quantity.
// Stochastic gradient in trace form (km_grad.cu): with X = [T alpha] in d_T (n x (p + 1)),
//   grad_j = 0.5 sum_c w_c x_c' dK_j x_c,   w_c = 1/p (probes), wa (alpha: -1, or -n / y'alpha
// for the profile likelihood),
// the same quantity as the reference's per-probe dots (stochasticgradient.jl:14-26) summed over
// the probes, split into the leaf terms <dK_j,l, G_l> (the leaf Gram matrices of X against the
// derivative entries, both formed in registers) and the landmark quadratic forms of the
// projections of X on [Phi dPhi_0 dPhi_1 dPhi_2] (one pass for the three parameters).
static int gradient_trace(km_handle* h, int64_t p, double wa, double* grad) {
  const Tree& t = h->tree;
  const int r = h->r;
  const int64_t n = t.n, kk = p + 1, W = 4 * r;
  cudaStream_t st = h->stream;
  int rc;
  const int64_t nlp = t.nleaf * leaf_dk_gram_parts(t);  // partial sums of the leaf term
  if ((rc = grow(h, &h->d_dPhi2, 2 * t.n * r)) || (rc = grow(h, &h->d_Sj3, 3 * r * r)) ||
      (rc = grow(h, &h->d_Sinv, r * r)) || (rc = grow(h, &h->d_VP4, (t.nleaf + 1) * kk * W)) ||
      (rc = grow(h, &h->d_gpart, 3 * nlp + 3 * (t.nleaf + 1) + 3)))
    return rc;
  if (h->mixed && ((rc = grow(h, &h->d_Phif, t.n * r)) || (rc = grow(h, &h->d_SinvF, r * r)) ||
                   (rc = grow(h, &h->d_Sj3F, 3 * r * r))))
    return rc;
  double* leafpart = h->d_gpart;
  double* lmpart = h->d_gpart + 3 * nlp;
  double* sums = lmpart + 3 * (t.nleaf + 1);
  // DerivativeHODLR (constructor.jl:66-95) for the three parameters: dK(X, P) and Sj = dK(P, P);
  // the dK leaves are evaluated inside the leaf kernel
  KLV(h, KM_PROF_OTHER, launch_small_gemm(h->d_SinvT, h->d_SinvT, r, 1, h->d_Sinv, st));  // S^{-1}
  for (int j = 0; j < 3; ++j)
    KLV(h, KM_PROF_EVAL, launch_eval_dense(h->d_lnd, r, h->d_lnd, r, h->kp, j, h->d_Sj3 + (int64_t)j * r * r, r, st));
  if (h->mixed) {
    KLV(h, KM_PROF_OTHER, launch_to_ff(h->d_Phi, P<ff>(h->d_Phif), t.n * r, st));
    KLV(h, KM_PROF_OTHER, launch_to_ff(h->d_Sinv, P<ff>(h->d_SinvF), (int64_t)r * r, st));
    KLV(h, KM_PROF_OTHER, launch_to_ff(h->d_Sj3, P<ff>(h->d_Sj3F), (int64_t)3 * r * r, st));
    KLV(h, KM_PROF_EVAL, launch_eval_dphi2<ff>(h->d_pts, h->d_lnd, h->d_pts3, h->d_lnd3, r, t, h->kp,
                                                P<ff>(h->d_dPhi2), st));
    // X in float pairs (d_U is free here: no product dK X is formed)
    KLV(h, KM_PROF_OTHER, launch_to_ff(h->d_T, P<ff>(h->d_U), n * kk, st));
    KLV(h, KM_PROF_LEAF_APPLY,
        launch_leaf_dk_gram<ff>(h->d_pts, h->d_pts3, h->kp, P<ff>(h->d_U), n, (int)p, wa, t, leafpart, st));
  } else {
    KLV(h, KM_PROF_EVAL, launch_eval_dphi2<double>(h->d_pts, h->d_lnd, nullptr, nullptr, r, t, h->kp, h->d_dPhi2, st));
    KLV(h, KM_PROF_LEAF_APPLY,
        launch_leaf_dk_gram<double>(h->d_pts, nullptr, h->kp, h->d_T, n, (int)p, wa, t, leafpart, st));
  }
  if (t.L > 0) {
    if (h->mixed) {
      KLV(h, KM_PROF_LEAF_APPLY,
          launch_leaf_proj3<ff>(P<ff>(h->d_Phif), P<ff>(h->d_dPhi2), r, t, P<ff>(h->d_U), n, h->d_VP4, (int)kk, st));
    } else {
      KLV(h, KM_PROF_LEAF_APPLY,
          launch_leaf_proj3<double>(h->d_Phi, h->d_dPhi2, r, t, h->d_T, n, h->d_VP4, (int)kk, st));
    }
    KLV(h, KM_PROF_LEAF_APPLY, launch_nugget_proj(h->d_pts, h->d_lnd, r, t, h->d_T, n, h->d_VP4, (int)kk, st));
    KLV(h, KM_PROF_OTHER, launch_proj_total(h->d_VP4, (int)W, t.nleaf, (int)kk, st));
    if (h->mixed)
      KLV(h, KM_PROF_LEAF_APPLY, launch_landmark<ff>(h->d_VP4, r, (int)kk, (int)p, wa, P<ff>(h->d_SinvF),
                                                     P<ff>(h->d_Sj3F), t.nleaf, lmpart, st));
    else
      KLV(h, KM_PROF_LEAF_APPLY, launch_landmark<double>(h->d_VP4, r, (int)kk, (int)p, wa, h->d_Sinv, h->d_Sj3,
                                                         t.nleaf, lmpart, st));
  } else {
    // a single leaf: no off-diagonal block, no landmark term
    KM_CUDA(h, cudaMemsetAsync(lmpart, 0, sizeof(double) * 3 * (t.nleaf + 1), st));
  }
  KLV(h, KM_PROF_OTHER, launch_grad_final(leafpart, nlp, lmpart, t.nleaf + 1, 0.5, sums, st));
  KM_CUDA(h, cudaMemcpyAsync(grad, sums, sizeof(double) * 3, cudaMemcpyDeviceToHost, st));
  return sync(h, "gradient");
}

static int nll_grad_impl(km_handle* h, const double* y, const double* probes, bool seeded, uint64_t seed,
                         int64_t nprobe, double* nll, double* grad, bool profile = false,
                         double* fisher = nullptr, double* ya_out = nullptr) {
  if (!h || !y || !nll || nprobe < 0 || (grad && (nprobe < 1 || (!probes && !seeded))) || (fisher && !grad))
    return fail(h, KM_ERR_BAD_ARG, "bad likelihood arguments");
  cudaSetDevice(h->cfg.device);
  if (!h->factorized) return fail(h, KM_ERR_STATE, "The HODLR matrix needs to be factorized for this.");
  if (grad && h->method != KM_METHOD_NYSTROM) return fail(h, KM_ERR_STATE, "This is only valid for Nystrom-block matrices.");
  const Tree& t = h->tree;
  const int64_t n = t.n;
  const int64_t p = grad ? nprobe : 0;
  const int64_t kk = p + 1;
  int rc;
  timer_start(h);
  if (kk > h->tcap) {
    h->tcap = 0;
    if ((rc = grow(h, &h->d_T, n * kk)) || (rc = grow(h, &h->d_U, n * kk)) || (rc = grow(h, &h->d_dots, kk)))
      return rc;
    h->tcap = kk;
  }
  if ((rc = ensure_vec(h, kk)) != KM_OK) return rc;
  cudaStream_t st = h->stream;
  double* alpha = h->d_T + n * p;  // last column
  KM_CUDA(h, cudaMemcpyAsync(alpha, y, sizeof(double) * n, cudaMemcpyHostToDevice, st));
  if ((rc = nested_solve(h, alpha, 1)) != KM_OK) return rc;
  double ld = 0.0;
  if (h->mixed)
    KLV(h, KM_PROF_OTHER, launch_logdet<ff>(P<ff>(h->d_Lf), t, P<ff>(h->d_L22), h->r, h->d_partial, kLogdetBlocks,
                                            h->d_scalar, st));
  else
    KLV(h, KM_PROF_OTHER, launch_logdet<double>(h->d_Lf, t, h->d_L22, h->r, h->d_partial, kLogdetBlocks,
                                                h->d_scalar, st));
  KM_CUDA(h, cudaMemcpyAsync(&ld, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, st));
  std::vector<double> a(n);
  KM_CUDA(h, cudaMemcpyAsync(a.data(), alpha, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  if ((rc = sync(h, "nll")) != KM_OK) return rc;
  double ya = 0.0;
  for (int64_t i = 0; i < n; ++i) ya += y[i] * a[i];
  if (profile && !(ya > 0.0)) return fail(h, KM_ERR_BAD_ARG, "y' K^-1 y is not positive (zero data?)");
  if (ya_out) *ya_out = ya;
  *nll = profile ? 0.5 * (ld + (double)n * std::log(ya)) : 0.5 * ld + 0.5 * ya;
  if (grad) {
    if (seeded)
      KLV(h, KM_PROF_OTHER, launch_rademacher(h->d_T, n, p, seed, st));
    else
      KM_CUDA(h, cudaMemcpyAsync(h->d_T, probes, sizeof(double) * n * p, cudaMemcpyHostToDevice, st));
    if ((rc = nested_bwd(h, h->d_T, (int)p)) != KM_OK) return rc;  // T = W'^{-1} V
    if (!fisher) {
      rc = gradient_trace(h, p, profile ? -(double)n / ya : -1.0, grad);
      if (rc != KM_OK) return rc;
      h->stats.grad_ms = timer_stop(h);
      return sync(h, "nll_grad");
    }
    if (fisher && (rc = grow(h, &h->d_A, 3 * n * p + 6 * p)) != KM_OK) return rc;  // + pairwise dots
    std::vector<double> dots(kk);
    for (int j = 0; j < 3; ++j) {
      if ((rc = derivative_apply(h, j, h->d_T, h->d_U, (int)kk)) != KM_OK) return rc;
      KLV(h, KM_PROF_OTHER, launch_col_dots(h->d_T, n, h->d_U, n, n, (int)kk, h->d_dots, st));
      KM_CUDA(h, cudaMemcpyAsync(dots.data(), h->d_dots, sizeof(double) * kk, cudaMemcpyDeviceToHost, st));
      if (fisher) {
        double* Aj = h->d_A + (int64_t)j * n * p;
        KM_CUDA(h, cudaMemcpyAsync(Aj, h->d_U, sizeof(double) * n * p, cudaMemcpyDeviceToDevice, st));
        if ((rc = nested_fwd(h, Aj, (int)p)) != KM_OK) return rc;  // A_j = W^{-1} dK_j T
      }
      if ((rc = sync(h, "grad")) != KM_OK) return rc;
      double tr = 0.0;
      for (int64_t c = 0; c < p; ++c) tr += dots[c];
      grad[j] = 0.5 * (tr / (double)p - (profile ? (double)n * dots[p] / ya : dots[p]));
    }
    if (fisher) {
      std::vector<double> fd(6 * p);
      double* d_fd = h->d_A + 3 * n * p;
      for (int j = 0, q = 0; j < 3; ++j)
        for (int k = j; k < 3; ++k, ++q)
          KLV(h, KM_PROF_OTHER, launch_col_dots(h->d_A + (int64_t)j * n * p, n, h->d_A + (int64_t)k * n * p, n, n,
                                                (int)p, d_fd + q * p, st));
      KM_CUDA(h, cudaMemcpyAsync(fd.data(), d_fd, sizeof(double) * 6 * p, cudaMemcpyDeviceToHost, st));
      if ((rc = sync(h, "fisher")) != KM_OK) return rc;
      for (int j = 0, q = 0; j < 3; ++j)
        for (int k = j; k < 3; ++k, ++q) {
          double m = 0.0;
          for (int64_t c = 0; c < p; ++c) m += fd[q * p + c];
          fisher[3 * j + k] = fisher[3 * k + j] = 0.5 * m / (double)p;
        }
    }
  }
  h->stats.grad_ms = timer_stop(h);
  return sync(h, "nll_grad");
}

int km_nll_grad(km_handle* h, const double* y, const double* probes, int64_t nprobe, double* nll,
                double* grad) {
  return nll_grad_impl(h, y, probes, false, 0, nprobe, nll, grad);
}

int km_nll_grad_seeded(km_handle* h, const double* y, int64_t nprobe, uint64_t seed, double* nll,
                       double* grad) {
  return nll_grad_impl(h, y, nullptr, true, seed, nprobe, nll, grad);
}

int km_grad_fisher(km_handle* h, const double* y, const double* probes, int64_t nprobe, double* nll,
                   double* grad, double* fisher) {
  if (!fisher) return fail(h, KM_ERR_BAD_ARG, "bad likelihood arguments");
  return nll_grad_impl(h, y, probes, false, 0, nprobe, nll, grad, false, fisher);
}

int km_grad_fisher_seeded(km_handle* h, const double* y, int64_t nprobe, uint64_t seed, double* nll,
                          double* grad, double* fisher) {
  if (!fisher) return fail(h, KM_ERR_BAD_ARG, "bad likelihood arguments");
  return nll_grad_impl(h, y, nullptr, true, seed, nprobe, nll, grad, false, fisher);
}

// Stochastic Hessian of the NLL (stoch_hessian, src/HODLR/src/stochastichessian.jl:117-147, with
// shuffle = false and profile = false): minus the stochastic Fisher matrix, plus for every pair
// j <= k the trace term 0.5 mean_v t'D2_jk t (t = W'^{-1} v, HODLR_hess_tr2 :79-89) where the
// second derivative is not identically zero, and minus half the solve term
// -u'dK_k K^{-1} dK_j u - u'dK_j K^{-1} dK_k u (+ u'D2_jk u), u = K^{-1} y (HODLR_hess_slv(_no2d)
// :3-13, :50-56), written with the symmetry of K^{-1} and dK_j.  The probes, W'^{-1} V and u come
// from the gradient and Fisher call.  With `profile` (stoch_hessian(..., profile = true), the
// Hessian of nlpl_hessian, maxlikfunctions.jl:120-136) NLL and gradient are the profile
// likelihood's and the solve term is HODLR_p_hess_slv's (stochastichessian.jl:15-31); a pair whose
// second derivative is identically zero, where the reference raises, takes its general path with
// a zero second derivative (no D2 term, no trace term).
static int hessian_impl(km_handle* h, const double* y, const double* probes, bool seeded, uint64_t seed,
                        int64_t nprobe, double* nll, double* grad, double* hess, bool profile = false) {
  if (!h || !hess || !grad || nprobe < 1) return fail(h, KM_ERR_BAD_ARG, "bad Hessian arguments");
  double F[9], ya = 0.0;
  int rc = nll_grad_impl(h, y, probes, seeded, seed, nprobe, nll, grad, profile, F, &ya);
  if (rc != KM_OK) return rc;
  const Tree& t = h->tree;
  const int64_t n = t.n, p = nprobe;
  cudaStream_t st = h->stream;
  const double* u = h->d_T + n * p;  // d_T = [W'^{-1} V | K^{-1} y]
  if ((rc = grow(h, &h->d_hA, 6 * n)) || (rc = grow(h, &h->d_hY, n * (p + 1))) ||
      (rc = grow(h, &h->d_hdots, p + 1 + 12)))
    return rc;
  double* a = h->d_hA;      // a_j = dK_j u
  double* b = a + 3 * n;    // b_j = K^{-1} a_j
  for (int j = 0; j < 3; ++j) {
    if ((rc = derivative_apply(h, j, u, a + j * n, 1)) != KM_OK) return rc;
    KM_CUDA(h, cudaMemcpyAsync(b + j * n, a + j * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    if ((rc = nested_solve(h, b + j * n, 1)) != KM_OK) return rc;
  }
  double* d_ab = h->d_hdots + p + 1;  // d_ab[3 j + k] = a_k . b_j, then d_ab[9 + j] = u . a_j
  for (int j = 0; j < 3; ++j)
    for (int k = 0; k < 3; ++k)
      KLV(h, KM_PROF_OTHER, launch_col_dots(a + k * n, n, b + j * n, n, n, 1, d_ab + 3 * j + k, st));
  for (int j = 0; j < 3; ++j) KLV(h, KM_PROF_OTHER, launch_col_dots(a + j * n, n, u, n, n, 1, d_ab + 9 + j, st));
  double ab[12];
  KM_CUDA(h, cudaMemcpyAsync(ab, d_ab, sizeof ab, cudaMemcpyDeviceToHost, st));
  if ((rc = sync(h, "hessian")) != KM_OK) return rc;
  std::vector<double> dd(p + 1);
  for (int j = 0; j < 3; ++j)
    for (int k = j; k < 3; ++k) {
      double sterm = -(ab[3 * j + k] + ab[3 * k + j]);
      double tr = 0.0;
      if (!d2_zero(h->kp.kid, j, k)) {
        if ((rc = deriv2_apply(h, j, k, h->d_T, h->d_hY, (int)(p + 1))) != KM_OK) return rc;
        KLV(h, KM_PROF_OTHER, launch_col_dots(h->d_T, n, h->d_hY, n, n, (int)(p + 1), h->d_hdots, st));
        KM_CUDA(h, cudaMemcpyAsync(dd.data(), h->d_hdots, sizeof(double) * (p + 1), cudaMemcpyDeviceToHost, st));
        if ((rc = sync(h, "hessian")) != KM_OK) return rc;
        for (int64_t c = 0; c < p; ++c) tr += dd[c];
        tr /= (double)p;
        sterm += dd[p];  // u' D2_jk u
      }
      // profile likelihood (HODLR_p_hess_slv, stochastichessian.jl:15-31): with dotm = y'u,
      // n (sterm / dotm + (u'dK_j u)(u'dK_k u) / dotm^2), since y'K^{-1} = u'
      if (profile) sterm = (double)n * (sterm / ya + ab[9 + j] * ab[9 + k] / (ya * ya));
      hess[3 * j + k] = hess[3 * k + j] = -F[3 * j + k] + 0.5 * tr - 0.5 * sterm;
    }
  return KM_OK;
}

int km_stoch_hessian(km_handle* h, const double* y, const double* probes, int64_t nprobe, double* nll,
                     double* grad, double* hess) {
  if (!probes) return fail(h, KM_ERR_BAD_ARG, "bad Hessian arguments");
  return hessian_impl(h, y, probes, false, 0, nprobe, nll, grad, hess);
}

int km_stoch_hessian_seeded(km_handle* h, const double* y, int64_t nprobe, uint64_t seed, double* nll,
                            double* grad, double* hess) {
  return hessian_impl(h, y, nullptr, true, seed, nprobe, nll, grad, hess);
}

int km_stoch_profile_hessian(km_handle* h, const double* y, const double* probes, int64_t nprobe, double* nll,
                             double* grad, double* hess) {
  if (!probes) return fail(h, KM_ERR_BAD_ARG, "bad Hessian arguments");
  return hessian_impl(h, y, probes, false, 0, nprobe, nll, grad, hess, true);
}

int km_stoch_profile_hessian_seeded(km_handle* h, const double* y, int64_t nprobe, uint64_t seed, double* nll,
                                    double* grad, double* hess) {
  return hessian_impl(h, y, nullptr, true, seed, nprobe, nll, grad, hess, true);
}

int km_profile_nll_grad(km_handle* h, const double* y, const double* probes, int64_t nprobe, double* nll,
                        double* grad) {
  return nll_grad_impl(h, y, probes, false, 0, nprobe, nll, grad, true);
}

int km_profile_nll_grad_seeded(km_handle* h, const double* y, int64_t nprobe, uint64_t seed, double* nll,
                               double* grad) {
  return nll_grad_impl(h, y, nullptr, true, seed, nprobe, nll, grad, true);
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Allocation-free solve (declared in include/kmhodlr.h).  The workspace is a fixed file-scope
// device array; host code obtains its device address once per device with cudaGetSymbolAddress
// (the host-side symbol itself is not a device address and must never be passed to a kernel).
// ---------------------------------------------------------------------------------------------
static constexpr size_t kNoAllocDoubles = KM_NOALLOC_SCRATCH_BYTES / sizeof(double);
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];
namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_dev[kMaxDevices] = {};
}  // namespace

// Columns the refinement of a mixed-precision handle can take in one allocation-free call: its
// residual norms come back to a host array of this fixed size on the stack.
static constexpr int64_t kNoAllocRefineCols = 256;

extern "C" int km_solve_noalloc(km_handle* h, const double* d_b, double* d_x, int64_t k) {
  if (!h || !d_b || !d_x || k < 1) return fail(h, KM_ERR_BAD_ARG, "bad solve arguments");
  const int dev = h->cfg.device;
  if (dev < 0 || dev >= kMaxDevices) return fail(h, KM_ERR_BAD_ARG, "device ordinal out of range");
  KM_CUDA(h, cudaSetDevice(dev));
  if (!h->factorized) return fail(h, KM_ERR_STATE, "No solves without factorization.");
  if (h->method != KM_METHOD_NYSTROM)
    return fail(h, KM_ERR_UNSUPPORTED,
                "km_solve_noalloc: only Nystrom handles; an ACA handle's solve sizes its workspace by the "
                "block ranks and grows it on the device, use km_solve_dev");
  const Tree& t = h->tree;
  const int64_t slots = t.nleaf + t.nnode;
  const int64_t vp = slots * h->r * k;
  const int64_t vd = std::max<int64_t>(t.nnode, 1) * 2 * h->r * k;
  const bool refining = h->mixed && h->cfg.refine_max_iter > 0;
  const bool in_place = d_x == d_b;
  // solve sweeps: VP, VG, VD; refinement: residual (n x k), its norms (2k) and, for an in-place
  // call, a copy of the right-hand sides (n x k)
  const int64_t need =
      2 * vp + vd + (refining ? t.n * k + 2 * k + (in_place ? t.n * k : 0) : 0);
  if (need > (int64_t)kNoAllocDoubles || (refining && k > kNoAllocRefineCols)) {
    char buf[320];
    snprintf(buf, sizeof buf,
             "km_solve_noalloc: %lld columns need %lld bytes of workspace but the fixed array holds "
             "%u bytes (refinement takes at most %lld columns); pass fewer columns per call",
             (long long)k, (long long)(need * sizeof(double)), (unsigned)KM_NOALLOC_SCRATCH_BYTES,
             (long long)kNoAllocRefineCols);
    return fail(h, KM_ERR_BAD_ARG, buf);
  }
  double* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_dev[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) return cuda_fail(h, e == cudaSuccess ? cudaErrorUnknown : e, "cudaGetSymbolAddress");
      g_noalloc_dev[dev] = (double*)p;
    }
    base = g_noalloc_dev[dev];
  }
  // run the ordinary solve (and refinement) on the fixed workspace; the handle's own workspace is
  // untouched
  double* const sv[3] = {h->d_VP, h->d_VG, h->d_VD};
  const bool prof = h->prof;
  h->prof = false;  // the profiler creates events on demand
  h->d_VP = base;
  h->d_VG = base + vp;
  h->d_VD = base + 2 * vp;
  double* res = base + 2 * vp + vd;
  double* rdots = res + t.n * k;
  double* bcopy = rdots + 2 * k;
  int rc = KM_OK;
  const double* b_keep = d_b;
  cudaError_t e = cudaSuccess;
  if (!in_place) {
    e = cudaMemcpyAsync(d_x, d_b, sizeof(double) * t.n * k, cudaMemcpyDeviceToDevice, h->stream);
  } else if (refining) {
    e = cudaMemcpyAsync(bcopy, d_b, sizeof(double) * t.n * k, cudaMemcpyDeviceToDevice, h->stream);
    b_keep = bcopy;
  }
  if (e != cudaSuccess) rc = cuda_fail(h, e, "cudaMemcpyAsync");
  if (rc == KM_OK) rc = nested_solve(h, d_x, (int)k);
  if (rc == KM_OK && refining) {
    double hdots[2 * kNoAllocRefineCols];
    rc = refine_with(h, b_keep, d_x, (int)k, res, rdots, hdots);
  }
  h->d_VP = sv[0];
  h->d_VG = sv[1];
  h->d_VD = sv[2];
  h->prof = prof;
  if (rc != KM_OK) return rc;
  return sync(h, "solve_noalloc");
}

// ---- memory management helpers for the batched and serving forms ----------------------------

extern "C" int km_trim(km_handle* h) {
  if (!h) return KM_ERR_BAD_ARG;
  cudaSetDevice(h->cfg.device);
  free_problem(h);
  return KM_OK;
}

// ---- k-d ordering of the input points (maxlikdata, src/HODLR/src/constructor.jl:171-181) -------

// Orders n points (AoS x, y, host) on the device; writes the permutation (perm[i] = original
// index of sorted position i) and, when pts_s is given, the sorted points and data.  Temporary
// device buffers are taken from the handle's budget and returned before the call ends.
static int kd_impl(km_handle* h, const double* pts, const double* data, int64_t n, int64_t leaf, int64_t* perm,
                   double* pts_s, double* data_s) {
  if (!h) return KM_ERR_BAD_ARG;
  if (!pts || n < 1 || leaf < 1 || n >= (int64_t(1) << 31) || (!perm && !pts_s) || (data && pts_s && !data_s))
    return fail(h, KM_ERR_BAD_ARG, "bad k-d ordering arguments");
  for (int64_t i = 0; i < 2 * n; ++i)
    if (!std::isfinite(pts[i])) return fail(h, KM_ERR_BAD_ARG, "a point coordinate is not finite");
  cudaSetDevice(h->cfg.device);
  double* d_pts = nullptr;
  double* d_data = nullptr;
  double* d_ps = nullptr;
  double* d_ds = nullptr;
  int64_t* d_perm = nullptr;
  unsigned char* d_scr = nullptr;
  auto release = [&] {
    dfree(h, d_pts);
    dfree(h, d_data);
    dfree(h, d_ps);
    dfree(h, d_ds);
    dfree(h, d_perm);
    dfree(h, d_scr);
  };
  const bool with_data = data && pts_s;
  int rc = dalloc(h, &d_pts, 2 * n);
  if (rc == KM_OK) rc = dalloc(h, &d_perm, n);
  if (rc == KM_OK) rc = dalloc(h, &d_scr, (int64_t)kd_scratch_bytes(n));
  if (rc == KM_OK && pts_s) rc = dalloc(h, &d_ps, 2 * n);
  if (rc == KM_OK && with_data) rc = dalloc(h, &d_data, n);
  if (rc == KM_OK && with_data) rc = dalloc(h, &d_ds, n);
  if (rc != KM_OK) {
    release();
    return rc;
  }
  cudaStream_t st = h->stream;
  std::string err;
  cudaError_t e = cudaMemcpyAsync(d_pts, pts, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && with_data) e = cudaMemcpyAsync(d_data, data, sizeof(double) * n, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && !kd_order_device(d_pts, n, leaf, d_perm, d_scr, st, &err)) {
    release();
    return fail(h, KM_ERR_CUDA, err);
  }
  if (e == cudaSuccess && pts_s) {
    launch_gather_sorted(d_pts, with_data ? d_data : nullptr, d_perm, n, d_ps, d_ds, st);
    e = cudaMemcpyAsync(pts_s, d_ps, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && with_data) e = cudaMemcpyAsync(data_s, d_ds, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess && perm) e = cudaMemcpyAsync(perm, d_perm, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  release();
  if (e != cudaSuccess) return cuda_fail(h, e, "k-d ordering");
  return KM_OK;
}

extern "C" int km_kd_order(km_handle* h, const double* pts, int64_t n, int64_t leaf, int64_t* perm) {
  return kd_impl(h, pts, nullptr, n, leaf, perm, nullptr, nullptr);
}

extern "C" int km_maxlikdata(km_handle* h, const double* pts, const double* data, int64_t n, int64_t leaf,
                             double* pts_sorted, double* data_sorted, int64_t* perm) {
  if (!pts_sorted) return fail(h, KM_ERR_BAD_ARG, "bad k-d ordering arguments");
  return kd_impl(h, pts, data, n, leaf, perm, pts_sorted, data_sorted);
}

// Mirrors the allocations of assemble_impl (Nystrom), ensure_vec, ensure_xy and nll_grad_impl
// with the trace-form gradient for one problem shape.
extern "C" int64_t km_estimate_bytes(int64_t n, int64_t rank, int level_kind, int64_t level, int64_t ncols,
                          int with_grad) {
  Tree t;
  std::string msg;
  if (rank < 1 || ncols < 0 || !build_tree(n, level_kind, level, &t, &msg)) return -1;
  const int64_t r = rank, k = std::max<int64_t>(ncols, 1);
  const int64_t nn = std::max<int64_t>(t.nnode, 1), slots = t.nleaf + t.nnode;
  int64_t kb = 0;
  for (int64_t j = 0; j < t.nleaf; ++j) kb += t.leaf_size(j) * t.leaf_size(j);
  auto d = [](int64_t c) { return 8 * std::max<int64_t>(c, 1); };
  int64_t b = d(2 * n) + d(2 * r) + d(4 * n) + d(4 * r) + d(r) + 2 * d(kb) + 2 * d(n * r) + d(t.nleaf * r) + d(slots * r * r) +
              4 * d(r * r) + 3 * d(nn * r * r) + d(nn * r) + d(nn * r * r) + d(nn * 2 * r * r) + d(nn * 5 * r * r) +
              4 * std::max<int64_t>(t.nleaf + t.nnode + 1, 1) + d(kLogdetBlocks) + d(4);
  b += 2 * d(slots * r * k) + d(nn * 2 * r * k);  // ensure_vec
  b += 2 * d(n * k);                              // ensure_xy
  if (leaf_tc_enabled() && leaf_chol_tc_supported(t, (int)r))  // slices of the tensor-core leaf stage
    b += leaf_chol_tc_scratch_bytes(t, (int)r);
  if (with_grad)  // trace-form gradient: [T alpha] and its float-pair copy, dK_j(X, P) for the scale
                  // and range, the float-pair Phi, S^{-1} and Sj, the projections, the partial sums
    b += 2 * d(n * k) + d(k) + d(2 * n * r) + d(n * r) + 2 * d(3 * r * r) + 2 * d(r * r) +
         d((t.nleaf + 1) * k * 4 * r) + d(3 * t.nleaf * leaf_dk_gram_parts(t) + 3 * t.nleaf + 6);
  return b;
}
