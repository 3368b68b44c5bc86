// C ABI of libkmhodlr: handle lifecycle, partition, and the orchestration of the device kernels.
// Each entry point mirrors one reference call (cited in include/kmhodlr.h).
#include <algorithm>
#include <mutex>
#include <cmath>
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
  double tol = 0.0;
  int64_t maxrank = 0;
  int r = 0;

  double* d_pts = nullptr;
  double* d_lnd = nullptr;
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
  double* d_Ct = nullptr;
  double* d_L22 = nullptr;
  double* d_Eref = nullptr;
  double* d_Etau = nullptr;
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
  // derivative HODLR (evaluated for one parameter at a time) and gradient workspaces
  int dk_param = -1;
  double* d_dK = nullptr;
  double* d_dPhi = nullptr;
  double* d_Sj = nullptr;
  double* d_GP = nullptr;
  double* d_GG = nullptr;
  int64_t gcap = 0;
  double* d_T = nullptr;
  double* d_U = nullptr;
  double* d_dots = nullptr;
  int64_t tcap = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaStream_t own_stream = nullptr;  // the handle's own stream (h->stream may be external)
  // profiler
  bool prof = false;
  struct Rec {
    int cls;
    cudaEvent_t a, b;
  };
  std::vector<Rec> pending;
  std::vector<cudaEvent_t> pool;
  double prof_ms[KM_PROF_COUNT] = {};
  int64_t prof_n[KM_PROF_COUNT] = {};
};

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
      return;
    }
  }
}

void free_problem(km_handle* h) {
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& a : h->allocs) cudaFree(a.first);
  h->allocs.clear();
  h->bytes = 0;
  h->d_pts = h->d_lnd = h->d_K = h->d_Lf = h->d_Phi = h->d_Q = h->d_tauleaf = h->d_R = nullptr;
  h->d_S = h->d_Sc = h->d_SinvT = h->d_Ct = h->d_L22 = h->d_Eref = h->d_Etau = nullptr;
  h->d_lndidx = nullptr;
  h->d_info = nullptr;
  h->d_partial = h->d_scalar = nullptr;
  h->d_VP = h->d_VG = h->d_VD = nullptr;
  h->vcap = 0;
  h->d_X = h->d_Y = nullptr;
  h->xcap = 0;
  h->dk_param = -1;
  h->d_dK = h->d_dPhi = h->d_Sj = h->d_GP = h->d_GG = h->d_T = h->d_U = h->d_dots = nullptr;
  h->gcap = h->tcap = 0;
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
  dfree(h, h->d_VP);
  dfree(h, h->d_VG);
  dfree(h, h->d_VD);
  h->d_VP = h->d_VG = h->d_VD = nullptr;
  h->vcap = 0;
  const int64_t slots = h->tree.nleaf + h->tree.nnode;
  int rc;
  if ((rc = dalloc(h, &h->d_VP, slots * h->r * k)) != KM_OK) return rc;
  if ((rc = dalloc(h, &h->d_VG, slots * h->r * k)) != KM_OK) return rc;
  if ((rc = dalloc(h, &h->d_VD, std::max<int64_t>(h->tree.nnode, 1) * 2 * h->r * k)) != KM_OK) return rc;
  h->vcap = k;
  return KM_OK;
}

int ensure_xy(km_handle* h, int64_t k) {
  if (k <= h->xcap) return KM_OK;
  dfree(h, h->d_X);
  dfree(h, h->d_Y);
  h->d_X = h->d_Y = nullptr;
  h->xcap = 0;
  int rc;
  if ((rc = dalloc(h, &h->d_X, h->tree.n * k)) != KM_OK) return rc;
  if ((rc = dalloc(h, &h->d_Y, h->tree.n * k)) != KM_OK) return rc;
  h->xcap = k;
  return KM_OK;
}

NodeMatsH node_mats(km_handle* h) { return NodeMatsH{h->d_Ct, h->d_L22, h->d_Eref, h->d_Etau, h->r}; }

// ---- factor sweeps on a device block X (n x k, ld = n), in place ---------------------------
int nested_fwd(km_handle* h, double* X, int k) {  // X <- W^{-1} X
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri(h->d_Lf, t, 0, X, 1, t.n, 0, X, 1, t.n, 0, k, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular solve kernel");
  if (t.L == 0) return check_launch(h, "fwd");
  NodeMatsH nm = node_mats(h);
  KLV(h, KM_PROF_LEAF_REFL, launch_leaf_proj(h->d_Q, h->d_tauleaf, h->r, t, X, t.n, h->d_VP, k, st));
  for (int l = 1; l <= t.L; ++l) KLV(h, KM_PROF_SWEEP, launch_up(t, nm, l, h->d_VP, h->d_VD, k, UP_FWD_, st));
  for (int l = t.L; l >= 1; --l) KLV(h, KM_PROF_SWEEP, launch_down(t, nm, l, h->d_VP, h->d_VG, h->d_VD, k, DN_FWD_, st));
  KLV(h, KM_PROF_LEAF_REFL, launch_leaf_expand(h->d_Q, h->d_tauleaf, h->r, t, h->d_VG, X, t.n, k, -1.0, st));
  return check_launch(h, "fwd");
}

int nested_bwd(km_handle* h, double* X, int k) {  // X <- W'^{-1} X
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  if (t.L > 0) {
    NodeMatsH nm = node_mats(h);
    KLV(h, KM_PROF_LEAF_REFL, launch_leaf_proj(h->d_Q, h->d_tauleaf, h->r, t, X, t.n, h->d_VP, k, st));
    for (int l = 1; l < t.L; ++l) KLV(h, KM_PROF_SWEEP, launch_up(t, nm, l, h->d_VP, h->d_VD, k, UP_PROJ_, st));
    for (int l = t.L; l >= 1; --l) KLV(h, KM_PROF_SWEEP, launch_down(t, nm, l, h->d_VP, h->d_VG, h->d_VD, k, DN_BWD_, st));
    KLV(h, KM_PROF_LEAF_REFL, launch_leaf_expand(h->d_Q, h->d_tauleaf, h->r, t, h->d_VG, X, t.n, k, -1.0, st));
  }
  if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri(h->d_Lf, t, 1, X, 1, t.n, 0, X, 1, t.n, 0, k, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular solve kernel");
  return check_launch(h, "bwd");
}

int nested_mul(km_handle* h, double* X, int k) {  // X <- W X
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  if (t.L > 0) {
    NodeMatsH nm = node_mats(h);
    KLV(h, KM_PROF_LEAF_REFL, launch_leaf_proj(h->d_Q, h->d_tauleaf, h->r, t, X, t.n, h->d_VP, k, st));
    for (int l = 1; l < t.L; ++l) KLV(h, KM_PROF_SWEEP, launch_up(t, nm, l, h->d_VP, h->d_VD, k, UP_PROJ_, st));
    for (int l = t.L; l >= 1; --l) KLV(h, KM_PROF_SWEEP, launch_down(t, nm, l, h->d_VP, h->d_VG, h->d_VD, k, DN_MUL_, st));
    KLV(h, KM_PROF_LEAF_REFL, launch_leaf_expand(h->d_Q, h->d_tauleaf, h->r, t, h->d_VG, X, t.n, k, 1.0, st));
  }
  if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri(h->d_Lf, t, 2, X, 1, t.n, 0, X, 1, t.n, 0, k, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular kernel");
  return check_launch(h, "mul");
}

int nested_mul_t(km_handle* h, double* X, int k) {  // X <- W' X
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri(h->d_Lf, t, 3, X, 1, t.n, 0, X, 1, t.n, 0, k, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular kernel");
  if (t.L == 0) return check_launch(h, "mul_t");
  NodeMatsH nm = node_mats(h);
  KLV(h, KM_PROF_LEAF_REFL, launch_leaf_proj(h->d_Q, h->d_tauleaf, h->r, t, X, t.n, h->d_VP, k, st));
  for (int l = 1; l <= t.L; ++l) KLV(h, KM_PROF_SWEEP, launch_up(t, nm, l, h->d_VP, h->d_VD, k, UP_MULT_, st));
  for (int l = t.L; l >= 1; --l) KLV(h, KM_PROF_SWEEP, launch_down(t, nm, l, h->d_VP, h->d_VG, h->d_VD, k, DN_MULT_, st));
  KLV(h, KM_PROF_LEAF_REFL, launch_leaf_expand(h->d_Q, h->d_tauleaf, h->r, t, h->d_VG, X, t.n, k, 1.0, st));
  return check_launch(h, "mul_t");
}

// Y = K X before factorisation (Nystrom blocks)
int nystrom_matvec(km_handle* h, const double* X, double* Y, int k) {
  const Tree& t = h->tree;
  cudaStream_t st = h->stream;
  NodeMatsH nm = node_mats(h);
  if (t.L > 0) {
    KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_phiT(h->d_Phi, h->r, t, X, t.n, h->d_VP, k, st));
    for (int l = 1; l < t.L; ++l) KLV(h, KM_PROF_SWEEP, launch_up(t, nm, l, h->d_VP, h->d_VD, k, UP_SUM_, st));
    for (int l = t.L; l >= 1; --l) KLV(h, KM_PROF_SWEEP, launch_down(t, nm, l, h->d_VP, h->d_VG, h->d_VD, k, DN_NYS_, st));
  } else {
    cudaMemsetAsync(h->d_VG, 0, sizeof(double) * h->r * k, st);
  }
  KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_nys_apply(h->d_K, h->d_Phi, h->d_Sc, h->r, t, X, t.n, h->d_VG, Y, t.n, k, st));
  return check_launch(h, "matvec");
}

int check_info(km_handle* h, int64_t count, const char* what) {
  std::vector<int> info(count);
  KM_CUDA(h, cudaMemcpy(info.data(), h->d_info, sizeof(int) * count, cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < count; ++i) {
    if (info[i] != 0) {
      char buf[160];
      snprintf(buf, sizeof buf, "PosDefException: %s %lld is not positive definite (pivot %d)",
               what, (long long)i, info[i]);
      return fail(h, KM_ERR_NOT_SPD, buf);
    }
  }
  return KM_OK;
}

// Y = dK_j X for the exact derivative of the Nystrom HODLR in parameter j (device pointers).
int derivative_apply(km_handle* h, int j, const double* X, double* Y, int k) {
  const Tree& t = h->tree;
  const int r = h->r;
  cudaStream_t st = h->stream;
  int rc;
  if (!h->d_dK) {
    int64_t kbytes = 0;
    for (int64_t q = 0; q < t.nleaf; ++q) kbytes += t.leaf_size(q) * t.leaf_size(q);
    if ((rc = dalloc(h, &h->d_dK, kbytes)) || (rc = dalloc(h, &h->d_dPhi, t.n * r)) ||
        (rc = dalloc(h, &h->d_Sj, r * r)))
      return rc;
  }
  if (k > h->gcap) {
    dfree(h, h->d_GP);
    dfree(h, h->d_GG);
    h->d_GP = h->d_GG = nullptr;
    h->gcap = 0;
    const int64_t slots = t.nleaf + t.nnode;
    if ((rc = dalloc(h, &h->d_GP, slots * 2 * r * k)) || (rc = dalloc(h, &h->d_GG, slots * 2 * r * k))) return rc;
    h->gcap = k;
  }
  if (h->dk_param != j) {
    // DerivativeHODLR (constructor.jl:66-95): dK leaves, dK(X, P) and Sj = dK(P, P)
    KLV(h, KM_PROF_EVAL, launch_eval_leaves(h->d_pts, t, h->kp, j, h->d_dK, st));
    KLV(h, KM_PROF_EVAL, launch_eval_phi(h->d_pts, h->d_lnd, r, t, h->kp, j, h->d_dPhi, st));
    KLV(h, KM_PROF_EVAL, launch_eval_dense(h->d_lnd, r, h->d_lnd, r, h->kp, j, h->d_Sj, r, st));
    h->dk_param = j;
  }
  NodeMatsH nm2{nullptr, nullptr, nullptr, nullptr, 2 * r};
  if (t.L > 0) {
    KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_dphiT(h->d_Phi, h->d_dPhi, r, t, X, t.n, h->d_GP, k, st));
    for (int l = 1; l < t.L; ++l) KLV(h, KM_PROF_SWEEP, launch_up(t, nm2, l, h->d_GP, nullptr, k, UP_SUM_, st));
    for (int l = t.L; l >= 1; --l) KLV(h, KM_PROF_SWEEP, launch_down(t, nm2, l, h->d_GP, h->d_GG, nullptr, k, DN_NYS_, st));
  } else {
    KM_CUDA(h, cudaMemsetAsync(h->d_GG, 0, sizeof(double) * 2 * r * k, st));
  }
  KLV(h, KM_PROF_LEAF_APPLY, launch_leaf_dnys_apply(h->d_dK, h->d_Phi, h->d_dPhi, h->d_Sc, h->d_Sj, r, t, X, t.n,
                                                    h->d_GG, Y, t.n, k, st));
  return check_launch(h, "derivative");
}

bool finite3(const double* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

}  // namespace

// ---------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------
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
  if (h->cfg.refine_max_iter <= 0) h->cfg.refine_max_iter = 30;
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
  if (cudaSetDevice(h->cfg.device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return KM_ERR_CUDA;
  }
  h->own_stream = h->stream;
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
  prof_resolve(h);
  for (auto e : h->pool) cudaEventDestroy(e);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
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
  if (method == KM_METHOD_ACA) return fail(h, KM_ERR_UNSUPPORTED, "ACA assembly is not built yet");
  // Nystrom checks (src/HODLR/src/constructor.jl:26-28)
  if (maxrank < 2) return fail(h, KM_ERR_BAD_ARG, "Please supply a fixed off-diagonal rank that is >=2.");
  const int64_t minleaf = t.m0;  // smallest leaf size
  if (maxrank >= minleaf - 1)
    return fail(h, KM_ERR_BAD_ARG, "Your nystrom rank is too big. Reduce the HODLR level or nystrom rank.");
  if (maxrank > kMaxNysRank) return fail(h, KM_ERR_UNSUPPORTED, "Nystrom rank above 80 is not supported");
  // Buffers are kept when the problem shape (n, levels, rank) is unchanged, so that repeated
  // assemblies (likelihood evaluations at new parameters) allocate nothing.
  const bool reuse = h->d_pts && h->tree.n == t.n && h->tree.L == t.L && h->r == (int)maxrank;
  if (!reuse) free_problem(h);
  h->tree = t;
  h->kp = KParams{kernel_id, params[0], params[1], params[2]};
  h->method = method;
  h->tol = tol;
  h->maxrank = maxrank;
  h->r = (int)maxrank;
  h->assembled = h->factorized = false;
  h->dk_param = -1;
  const int r = h->r;
  int64_t kbytes = 0;
  for (int64_t j = 0; j < t.nleaf; ++j) kbytes += t.leaf_size(j) * t.leaf_size(j);
  int rc;
  if (!reuse &&
      ((rc = dalloc(h, &h->d_pts, 2 * n)) || (rc = dalloc(h, &h->d_lnd, 2 * r)) ||
       (rc = dalloc(h, &h->d_lndidx, r)) || (rc = dalloc(h, &h->d_K, kbytes)) ||
       (rc = dalloc(h, &h->d_Lf, kbytes)) || (rc = dalloc(h, &h->d_Phi, n * r)) ||
       (rc = dalloc(h, &h->d_Q, n * r)) || (rc = dalloc(h, &h->d_tauleaf, t.nleaf * r)) ||
       (rc = dalloc(h, &h->d_R, (t.nleaf + t.nnode) * r * r)) || (rc = dalloc(h, &h->d_S, r * r)) ||
       (rc = dalloc(h, &h->d_Sc, r * r)) || (rc = dalloc(h, &h->d_SinvT, r * r)) ||
       (rc = dalloc(h, &h->d_Ct, std::max<int64_t>(t.nnode, 1) * r * r)) ||
       (rc = dalloc(h, &h->d_L22, std::max<int64_t>(t.nnode, 1) * r * r)) ||
       (rc = dalloc(h, &h->d_Eref, std::max<int64_t>(t.nnode, 1) * r * r)) ||
       (rc = dalloc(h, &h->d_Etau, std::max<int64_t>(t.nnode, 1) * r)) ||
       (rc = dalloc(h, &h->d_info, t.nleaf + t.nnode + 1)) ||
       (rc = dalloc(h, &h->d_partial, kLogdetBlocks)) || (rc = dalloc(h, &h->d_scalar, 4)))) {
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
  KLV(h, KM_PROF_EVAL, launch_eval_leaves(h->d_pts, t, h->kp, -1, h->d_K, st));
  KLV(h, KM_PROF_EVAL, launch_eval_phi(h->d_pts, h->d_lnd, r, t, h->kp, -1, h->d_Phi, st));
  KLV(h, KM_PROF_EVAL, launch_eval_dense(h->d_lnd, r, h->d_lnd, r, h->kp, -1, h->d_S, r, st));
  KM_CUDA(h, cudaMemcpyAsync(h->d_Sc, h->d_S, sizeof(double) * r * r, cudaMemcpyDeviceToDevice, st));
  if (!KL(h, KM_PROF_OTHER, launch_chol_small(h->d_Sc, r, h->d_info + t.nleaf + t.nnode, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "rank too large for the landmark Cholesky");
  KLV(h, KM_PROF_OTHER, launch_tri_inv_t(h->d_Sc, r, h->d_SinvT, st));
  if ((rc = check_launch(h, "assemble")) != KM_OK) return rc;
  h->stats.assemble_ms = timer_stop(h);
  if ((rc = sync(h, "assemble")) != KM_OK) return rc;
  int sinfo = 0;
  KM_CUDA(h, cudaMemcpy(&sinfo, h->d_info + t.nleaf + t.nnode, sizeof(int), cudaMemcpyDeviceToHost));
  if (sinfo != 0) return fail(h, KM_ERR_NOT_SPD, "PosDefException: landmark matrix K(P, P) is not positive definite");
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

int km_factorize(km_handle* h) {
  if (!h) return KM_ERR_BAD_ARG;
  cudaSetDevice(h->cfg.device);
  if (!h->assembled) return fail(h, KM_ERR_STATE, "assemble first");
  const Tree& t = h->tree;
  const int r = h->r;
  cudaStream_t st = h->stream;
  int rc;
  timer_start(h);
  KM_CUDA(h, cudaMemsetAsync(h->d_info, 0, sizeof(int) * (t.nleaf + t.nnode), st));
  if (!KL(h, KM_PROF_LEAF_CHOL, launch_leaf_chol(h->d_K, h->d_Lf, t, h->d_info, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the leaf Cholesky kernel");
  // A = L^{-1} Phi on every leaf, then Householder QR of each leaf panel
  KM_CUDA(h, cudaMemcpyAsync(h->d_Q, h->d_Phi, sizeof(double) * t.n * r, cudaMemcpyDeviceToDevice, st));
  if (!KL(h, KM_PROF_LEAF_TRI, launch_leaf_tri(h->d_Lf, t, 0, h->d_Q, r, 0, 1, h->d_Q, r, 0, 1, r, st)))
    return fail(h, KM_ERR_UNSUPPORTED, "leaf too large for the triangular solve kernel");
  if (t.L > 0) {
    KLV(h, KM_PROF_LEAF_QR, launch_leaf_qr(h->d_Q, r, t, h->d_tauleaf, h->d_R, st));
    for (int l = 1; l <= t.L; ++l)
      KLV(h, KM_PROF_NODE, launch_node_factor(h->d_R, h->d_SinvT, r, l, t, h->d_Ct, h->d_L22, h->d_Eref,
                                              h->d_Etau, h->d_info + t.nleaf, st));
  }
  if ((rc = check_launch(h, "factorize")) != KM_OK) return rc;
  h->stats.factorize_ms = timer_stop(h);
  if ((rc = sync(h, "factorize")) != KM_OK) return rc;
  if ((rc = check_info(h, t.nleaf, "leaf")) != KM_OK) return rc;
  {
    std::vector<int> info(t.nnode);
    if (t.nnode > 0)
      KM_CUDA(h, cudaMemcpy(info.data(), h->d_info + t.nleaf, sizeof(int) * t.nnode, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < t.nnode; ++i)
      if (info[i]) return fail(h, KM_ERR_NOT_SPD, "PosDefException: a low-rank capacitance block is not positive definite");
  }
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

int km_solve_dev(km_handle* h, const double* d_b, double* d_x, int64_t k) {
  if (!h || !d_b || !d_x || k < 1) return fail(h, KM_ERR_BAD_ARG, "bad solve arguments");
  cudaSetDevice(h->cfg.device);
  if (!h->factorized) return fail(h, KM_ERR_STATE, "No solves without factorization.");
  int rc;
  if ((rc = ensure_vec(h, k)) != KM_OK) return rc;
  timer_start(h);
  if (d_x != d_b)
    KM_CUDA(h, cudaMemcpyAsync(d_x, d_b, sizeof(double) * h->tree.n * k, cudaMemcpyDeviceToDevice, h->stream));
  if ((rc = nested_fwd(h, d_x, (int)k)) != KM_OK) return rc;
  if ((rc = nested_bwd(h, d_x, (int)k)) != KM_OK) return rc;
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
  KLV(h, KM_PROF_OTHER, launch_logdet(h->d_Lf, h->tree, h->d_L22, h->r, h->d_partial, kLogdetBlocks, h->d_scalar, h->stream));
  h->stats.kernel_launches += 1;  // the logdet runs a partial and a final reduction kernel
  int rc;
  if ((rc = check_launch(h, "logdet")) != KM_OK) return rc;
  KM_CUDA(h, cudaMemcpyAsync(out, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  h->stats.logdet_ms = timer_stop(h);
  return sync(h, "logdet");
}

int km_block_ranks(km_handle* h, int64_t* out) {
  if (!h || !out) return fail(h, KM_ERR_BAD_ARG, "null");
  if (!h->assembled) return fail(h, KM_ERR_STATE, "assemble first");
  for (int64_t q = 0; q < h->tree.nnode; ++q) out[q] = h->r;
  return KM_OK;
}

int km_aca_pivots(km_handle* h, int64_t, int64_t, int64_t*, int64_t*, int64_t*) {
  return fail(h, KM_ERR_UNSUPPORTED, "ACA assembly is not built yet");
}

int km_block_factors(km_handle* h, int64_t, double*, double*) {
  return fail(h, KM_ERR_UNSUPPORTED, "block factor export is not built yet");
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
int km_nll_grad(km_handle* h, const double* y, const double* probes, int64_t nprobe, double* nll,
                double* grad) {
  if (!h || !y || !nll || nprobe < 0 || (grad && (nprobe < 1 || !probes)))
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
    dfree(h, h->d_T);
    dfree(h, h->d_U);
    dfree(h, h->d_dots);
    h->d_T = h->d_U = h->d_dots = nullptr;
    h->tcap = 0;
    if ((rc = dalloc(h, &h->d_T, n * kk)) || (rc = dalloc(h, &h->d_U, n * kk)) || (rc = dalloc(h, &h->d_dots, kk)))
      return rc;
    h->tcap = kk;
  }
  if ((rc = ensure_vec(h, kk)) != KM_OK) return rc;
  cudaStream_t st = h->stream;
  double* alpha = h->d_T + n * p;  // last column
  KM_CUDA(h, cudaMemcpyAsync(alpha, y, sizeof(double) * n, cudaMemcpyHostToDevice, st));
  if ((rc = nested_fwd(h, alpha, 1)) != KM_OK) return rc;
  if ((rc = nested_bwd(h, alpha, 1)) != KM_OK) return rc;
  double ld = 0.0;
  KLV(h, KM_PROF_OTHER, launch_logdet(h->d_Lf, t, h->d_L22, h->r, h->d_partial, kLogdetBlocks, h->d_scalar, st));
  KM_CUDA(h, cudaMemcpyAsync(&ld, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, st));
  std::vector<double> a(n);
  KM_CUDA(h, cudaMemcpyAsync(a.data(), alpha, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  if ((rc = sync(h, "nll")) != KM_OK) return rc;
  double ya = 0.0;
  for (int64_t i = 0; i < n; ++i) ya += y[i] * a[i];
  *nll = 0.5 * ld + 0.5 * ya;
  if (grad) {
    KM_CUDA(h, cudaMemcpyAsync(h->d_T, probes, sizeof(double) * n * p, cudaMemcpyHostToDevice, st));
    if ((rc = nested_bwd(h, h->d_T, (int)p)) != KM_OK) return rc;  // T = W'^{-1} V
    std::vector<double> dots(kk);
    for (int j = 0; j < 3; ++j) {
      if ((rc = derivative_apply(h, j, h->d_T, h->d_U, (int)kk)) != KM_OK) return rc;
      KLV(h, KM_PROF_OTHER, launch_col_dots(h->d_T, n, h->d_U, n, n, (int)kk, h->d_dots, st));
      KM_CUDA(h, cudaMemcpyAsync(dots.data(), h->d_dots, sizeof(double) * kk, cudaMemcpyDeviceToHost, st));
      if ((rc = sync(h, "grad")) != KM_OK) return rc;
      double tr = 0.0;
      for (int64_t c = 0; c < p; ++c) tr += dots[c];
      grad[j] = 0.5 * (tr / (double)p - dots[p]);
    }
  }
  h->stats.grad_ms = timer_stop(h);
  return sync(h, "nll_grad");
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

extern "C" int km_solve_noalloc(km_handle* h, const double* d_b, double* d_x, int64_t k) {
  if (!h || !d_b || !d_x || k < 1) return fail(h, KM_ERR_BAD_ARG, "bad solve arguments");
  const int dev = h->cfg.device;
  if (dev < 0 || dev >= kMaxDevices) return fail(h, KM_ERR_BAD_ARG, "device ordinal out of range");
  KM_CUDA(h, cudaSetDevice(dev));
  if (!h->factorized) return fail(h, KM_ERR_STATE, "No solves without factorization.");
  const Tree& t = h->tree;
  const int64_t slots = t.nleaf + t.nnode;
  const int64_t vp = slots * h->r * k;
  const int64_t need = 2 * vp + std::max<int64_t>(t.nnode, 1) * 2 * h->r * k;
  if (need > (int64_t)kNoAllocDoubles) {
    char buf[256];
    snprintf(buf, sizeof buf,
             "km_solve_noalloc: %lld columns need %lld bytes of workspace but the fixed array holds "
             "%u bytes; pass fewer columns per call",
             (long long)k, (long long)(need * sizeof(double)), (unsigned)KM_NOALLOC_SCRATCH_BYTES);
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
  // run the ordinary solve sweeps on the fixed workspace; the handle's own workspace is untouched
  double* const sv[3] = {h->d_VP, h->d_VG, h->d_VD};
  const bool prof = h->prof;
  h->prof = false;  // the profiler creates events on demand
  h->d_VP = base;
  h->d_VG = base + vp;
  h->d_VD = base + 2 * vp;
  int rc = KM_OK;
  if (d_x != d_b) {
    cudaError_t e = cudaMemcpyAsync(d_x, d_b, sizeof(double) * t.n * k, cudaMemcpyDeviceToDevice, h->stream);
    if (e != cudaSuccess) rc = cuda_fail(h, e, "cudaMemcpyAsync");
  }
  if (rc == KM_OK) rc = nested_fwd(h, d_x, (int)k);
  if (rc == KM_OK) rc = nested_bwd(h, d_x, (int)k);
  h->d_VP = sv[0];
  h->d_VG = sv[1];
  h->d_VD = sv[2];
  h->prof = prof;
  if (rc != KM_OK) return rc;
  return sync(h, "solve_noalloc");
}
