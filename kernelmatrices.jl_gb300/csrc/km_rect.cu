// RKernelHODLR: the recursive, not necessarily symmetric or square, HODLR approximation of a
// kernel matrix K(x1, x2) that only supports products (src/HODLR/src/constructor.jl:130-161,
// src/HODLR/src/structstypes.jl:22-27, product src/HODLR/src/baseoverloads.jl:301-318).
//
// At every level the row range is split at floor(len1/2) and the column range at floor(len2/2);
// the off-diagonal blocks A12 (first rows, second columns) and A21 (second rows, first columns)
// are compressed separately by ACA, and after `levels` splits the diagonal blocks are kept dense.
// The points x1 and x2 are stored one after the other, so every block is a block of the kernel
// matrix of the concatenated points and the ACA kernels of the symmetric path compress it
// unchanged (the nugget term compares coordinates, so it applies where x1 and x2 share a point,
// as in the reference).  Blocks are numbered in the reference's recursive order: A12, A21, then
// the blocks of A11, then those of A22.
//
// Product y = R x (x: n2 x k, y: n1 x k): the dense leaves write their rows of y, then one depth
// at a time (rows are disjoint within a depth) every block adds U (V' x): V' x by chunks of rows
// of V (partial sums in a fixed order, no atomics), then U t by chunks of rows of U.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "km_kernels.h"

using namespace km;

namespace {

constexpr int kRectChunk = 2048;  // rows of V or U per CTA in the block products

struct RLeaf {
  int64_t row0, m1, col0, m2, off;  // rows of x1 / columns of x2 (unshifted), K at d_leafK + off
};
struct RChunk {                     // rows [i0, i0 + len) of block b (of V or of U)
  int b;
  int64_t i0, len;
};
// Workspace slots for k right-hand sides: block b's V' x partials start at part0 * k (chunk h,
// column c, rank index q at part0 * k + (h k + c) rank + q), its t values at t * k (column c,
// index q at t * k + c rank + q); part0 and t are the offsets for one column.
struct RBlockDev {                  // what the product kernels need of a block
  int64_t row0, nro, col0, ncl;     // unshifted row / column starts
  int64_t offU, offV;
  int rank;
  int64_t t, part0;
  int nchv;                         // chunks of V
};

constexpr int kLeafStage = 4096;  // columns of x staged in shared memory at a time

// y[row0 + i, c] = sum_j K[i + j m1] x[col0 + j, c]: grid (leaves, k), thread per row; x is staged
// kLeafStage entries at a time and each y entry belongs to one thread
__global__ void k_rleaf_apply(const RLeaf* __restrict__ leaves, const double* __restrict__ K,
                              const double* __restrict__ X, int64_t ldx, double* __restrict__ Y, int64_t ldy) {
  __shared__ double xs[kLeafStage];
  const RLeaf lf = leaves[blockIdx.x];
  const int c = blockIdx.y;
  const double* A = K + lf.off;
  for (int64_t j0 = 0; j0 < lf.m2; j0 += kLeafStage) {
    const int64_t nj = (lf.m2 - j0 < kLeafStage) ? lf.m2 - j0 : kLeafStage;
    __syncthreads();
    for (int64_t j = threadIdx.x; j < nj; j += blockDim.x) xs[j] = X[c * ldx + lf.col0 + j0 + j];
    __syncthreads();
    for (int64_t i = threadIdx.x; i < lf.m1; i += blockDim.x) {
      double acc = 0.0;
      for (int64_t j = 0; j < nj; ++j) acc += A[i + (j0 + j) * lf.m1] * xs[j];
      double* yp = Y + c * ldy + lf.row0 + i;
      *yp = (j0 == 0) ? acc : *yp + acc;
    }
  }
}

// V' x partial sums: grid (V chunks, k), one warp per rank index q
__global__ void k_rblock_vt(const RChunk* __restrict__ chunks, const RBlockDev* __restrict__ blocks,
                            const double* __restrict__ P, const double* __restrict__ X, int64_t ldx,
                            double* __restrict__ part, int k) {
  const RChunk ch = chunks[blockIdx.x];
  const RBlockDev b = blocks[ch.b];
  const int c = blockIdx.y;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const double* V = P + b.offV;
  const double* x = X + c * ldx + b.col0;
  const int64_t h = ch.i0 / kRectChunk;
  double* out = part + b.part0 * k + (h * k + c) * b.rank;
  for (int q = w; q < b.rank; q += nw) {
    double acc = 0.0;
    for (int64_t j = ch.i0 + lane; j < ch.i0 + ch.len; j += 32) acc += V[j + q * b.ncl] * x[j];
    acc = warp_sum(acc);
    if (lane == 0) out[q] = acc;
  }
}

// t = sum of the V chunks' partials in chunk order: grid (blocks at this depth, k)
__global__ void k_rblock_tsum(const int* __restrict__ ids, const RBlockDev* __restrict__ blocks,
                              const double* __restrict__ part, double* __restrict__ T, int k) {
  const RBlockDev b = blocks[ids[blockIdx.x]];
  const int c = blockIdx.y;
  for (int q = threadIdx.x; q < b.rank; q += blockDim.x) {
    double s = 0.0;
    for (int h = 0; h < b.nchv; ++h) s += part[b.part0 * k + ((int64_t)h * k + c) * b.rank + q];
    T[b.t * k + (int64_t)c * b.rank + q] = s;
  }
}

// y[row0 + i, c] += sum_q U[i + q nro] t[q]: grid (U chunks, k), thread per row
__global__ void k_rblock_u(const RChunk* __restrict__ chunks, const RBlockDev* __restrict__ blocks,
                           const double* __restrict__ P, const double* __restrict__ T, double* __restrict__ Y,
                           int64_t ldy, int k) {
  extern __shared__ double ts[];
  const RChunk ch = chunks[blockIdx.x];
  const RBlockDev b = blocks[ch.b];
  const int c = blockIdx.y;
  for (int q = threadIdx.x; q < b.rank; q += blockDim.x) ts[q] = T[b.t * k + (int64_t)c * b.rank + q];
  __syncthreads();
  const double* U = P + b.offU;
  for (int64_t i = ch.i0 + threadIdx.x; i < ch.i0 + ch.len; i += blockDim.x) {
    double acc = 0.0;
    for (int q = 0; q < b.rank; ++q) acc += U[i + q * b.nro] * ts[q];
    Y[c * ldy + b.row0 + i] += acc;
  }
}

thread_local std::string g_create_error;

}  // namespace

struct km_rhodlr {
  km_config cfg{};
  cudaStream_t st = nullptr;
  std::string err;
  int64_t n1 = 0, n2 = 0;
  int levels = 0;
  KParams kp{};
  std::vector<AcaBlock> blk;
  std::vector<int> depth;
  std::vector<int> rank;
  std::vector<RLeaf> leaves;
  // per depth: block ids, V chunks, U chunks (device copies below)
  std::vector<std::vector<int>> ids_at;
  std::vector<std::vector<RChunk>> vch_at, uch_at;
  int maxrank_seen = 0;
  int64_t nparts = 0, nt = 0;  // partial and t slots per right-hand-side column
  std::vector<void*> allocs;
  double* d_pts = nullptr;
  double* d_panels = nullptr;
  uint8_t* d_flags = nullptr;
  int* d_piv = nullptr;
  int* d_rank = nullptr;
  int* d_status = nullptr;
  AcaBlock* d_blk = nullptr;
  double* d_scr = nullptr;
  double* d_leafK = nullptr;
  RLeaf* d_leaves = nullptr;
  RBlockDev* d_bdev = nullptr;
  std::vector<int*> d_ids;
  std::vector<RChunk*> d_vch, d_uch;
  // product workspaces (grown)
  double* d_X = nullptr;
  double* d_Y = nullptr;
  double* d_part = nullptr;
  double* d_T = nullptr;
  int64_t kcap = 0;
};

namespace {

template <typename T>
bool ralloc(km_rhodlr* R, T** p, int64_t count) {
  void* q = nullptr;
  const cudaError_t e = cudaMalloc(&q, (size_t)std::max<int64_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) {
    cudaGetLastError();
    R->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return false;
  }
  R->allocs.push_back(q);
  *p = static_cast<T*>(q);
  return true;
}

void rfree(km_rhodlr* R, void* p) {
  if (!p) return;
  auto it = std::find(R->allocs.begin(), R->allocs.end(), p);
  if (it != R->allocs.end()) {
    cudaFree(p);
    R->allocs.erase(it);
  }
}

// the recursive block structure of constructor.jl:130-161 (0-based, unshifted columns)
void build_blocks(km_rhodlr* R, int64_t r0, int64_t l1, int64_t c0, int64_t l2, int lv, int d, int64_t maxrank) {
  const int64_t m1 = l1 / 2, m2 = l2 / 2;
  auto add = [&](int64_t a, int64_t na, int64_t b, int64_t nb) {
    AcaBlock q{};
    q.row0 = a;
    q.nro = na;
    q.col0 = R->n1 + b;  // columns index x2, stored after x1
    q.ncl = nb;
    const int64_t minsz = std::min(na, nb);
    q.maxsz = (int)(maxrank == 0 ? minsz : std::min<int64_t>(maxrank, minsz));
    q.grid = minsz >= kAcaGridMin ? 1 : 0;
    R->blk.push_back(q);
    R->depth.push_back(d);
  };
  add(r0, m1, c0 + m2, l2 - m2);  // A12
  add(r0 + m1, l1 - m1, c0, m2);  // A21
  if (lv == 1) {
    R->leaves.push_back(RLeaf{r0, m1, c0, m2, 0});
    R->leaves.push_back(RLeaf{r0 + m1, l1 - m1, c0 + m2, l2 - m2, 0});
  } else {
    build_blocks(R, r0, m1, c0, m2, lv - 1, d + 1, maxrank);
    build_blocks(R, r0 + m1, l1 - m1, c0 + m2, l2 - m2, lv - 1, d + 1, maxrank);
  }
}

int rfail(km_rhodlr* R, int code, const std::string& msg) {
  R->err = msg;
  return code;
}

bool ensure_k(km_rhodlr* R, int64_t k) {
  if (k <= R->kcap) return true;
  rfree(R, R->d_X);
  rfree(R, R->d_Y);
  rfree(R, R->d_part);
  rfree(R, R->d_T);
  R->d_X = R->d_Y = R->d_part = R->d_T = nullptr;
  R->kcap = 0;
  if (!ralloc(R, &R->d_X, R->n2 * k) || !ralloc(R, &R->d_Y, R->n1 * k) || !ralloc(R, &R->d_part, R->nparts * k) ||
      !ralloc(R, &R->d_T, R->nt * k))
    return false;
  R->kcap = k;
  return true;
}

void destroy(km_rhodlr* R) {
  if (!R) return;
  for (void* p : R->allocs) cudaFree(p);
  R->allocs.clear();
  if (R->st) cudaStreamDestroy(R->st);
  delete R;
}

}  // namespace

extern "C" const char* km_rhodlr_create_error(void) { return g_create_error.c_str(); }
extern "C" const char* km_rhodlr_last_error(const km_rhodlr* R) { return R ? R->err.c_str() : "null"; }

extern "C" int km_rhodlr_create(const km_config* cfg, const double* x1, int64_t n1, const double* x2, int64_t n2,
                                int kernel_id, const double* params, int nparams, double tol, int64_t maxrank,
                                int level_kind, int64_t level, km_rhodlr** out) {
  g_create_error.clear();
  auto bad = [&](int code, const std::string& msg) {
    g_create_error = msg;
    return code;
  };
  if (!cfg || !x1 || !x2 || !out || !params || nparams < 3 || n1 < 1 || n2 < 1 || maxrank < 0 || !(tol >= 0.0) ||
      (kernel_id != KM_KERNEL_RATQUAD && kernel_id != KM_KERNEL_MATERN32))
    return bad(KM_ERR_BAD_ARG, "bad RKernelHODLR arguments");
  *out = nullptr;
  // LogLevel(lv) -> FixedLevel(floor(log2(min(n1, n2))) - lv) (constructor.jl:134-137)
  const int64_t mn = std::min(n1, n2);
  int fl = 0;
  while ((mn >> (fl + 1)) > 0) ++fl;
  int64_t lv = level_kind == KM_LEVEL_LOG ? fl - level : level;
  if (level_kind != KM_LEVEL_FIXED && level_kind != KM_LEVEL_LOG) return bad(KM_ERR_BAD_ARG, "bad level kind");
  if (lv < 0) return bad(KM_ERR_BAD_ARG, "the level resolves to a negative depth");
  if (lv > 40 || (lv > 0 && (mn >> (lv - 1)) < 2))
    return bad(KM_ERR_BAD_ARG, "too many levels for the matrix size (a split would leave an empty block)");
  int dev = 0;
  if (cudaGetDeviceCount(&dev) != cudaSuccess || dev <= cfg->device || cfg->device < 0) {
    cudaGetLastError();
    return bad(KM_ERR_CUDA, "no such CUDA device");
  }
  cudaSetDevice(cfg->device);
  auto* R = new km_rhodlr;
  R->cfg = *cfg;
  R->n1 = n1;
  R->n2 = n2;
  R->levels = (int)lv;
  R->kp = make_kparams(kernel_id, params[0], params[1], params[2]);
  if (cudaStreamCreateWithFlags(&R->st, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    destroy(R);
    return bad(KM_ERR_CUDA, "cudaStreamCreate failed");
  }
  if (lv == 0) {
    R->leaves.push_back(RLeaf{0, n1, 0, n2, 0});
  } else {
    build_blocks(R, 0, n1, 0, n2, (int)lv, 0, maxrank);
  }
  int64_t koff = 0;
  for (auto& lf : R->leaves) {
    if (lf.m1 * lf.m2 >= (int64_t(1) << 31)) {
      destroy(R);
      return bad(KM_ERR_UNSUPPORTED, "a dense diagonal block has 2^31 entries or more; use more levels");
    }
    lf.off = koff;
    koff += lf.m1 * lf.m2;
  }
  // ACA panels: capacity as in the symmetric ACA assembly, bounded by the block sizes
  const int nb = (int)R->blk.size();
  int64_t offP = 0, offF = 0, offV = 0;
  int maxcap = 0;
  size_t freeb = 0, totb = 0;
  cudaMemGetInfo(&freeb, &totb);
  const double frac = cfg->hbm_budget_fraction > 0.0 ? cfg->hbm_budget_fraction : 0.8;
  int capmax = 256;
  for (int c = kAcaMaxCap; c > 256; c >>= 1) {
    int64_t tot = 0;
    for (const auto& b : R->blk) tot += (b.nro + b.ncl) * (int64_t)std::min(b.maxsz, c);
    if ((double)tot * 8.0 <= 0.4 * frac * (double)totb) {
      capmax = c;
      break;
    }
  }
  for (auto& b : R->blk) {
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
  int gmax = 0;
  for (const auto& b : R->blk)
    if (b.grid) gmax = std::max(gmax, b.cap);
  const int64_t ntot = n1 + n2;
  if (!ralloc(R, &R->d_pts, 2 * ntot) || !ralloc(R, &R->d_leafK, koff) ||
      (nb > 0 && (!ralloc(R, &R->d_panels, offP) || !ralloc(R, &R->d_flags, offF) || !ralloc(R, &R->d_piv, 2 * offV) ||
                  !ralloc(R, &R->d_rank, nb) || !ralloc(R, &R->d_status, nb) || !ralloc(R, &R->d_blk, nb))) ||
      (gmax > 0 && !ralloc(R, &R->d_scr, aca_grid_scratch(gmax))) ||
      !ralloc(R, &R->d_leaves, (int64_t)R->leaves.size())) {
    g_create_error = R->err;
    destroy(R);
    return KM_ERR_OOM;
  }
  cudaStream_t st = R->st;
  cudaMemcpyAsync(R->d_pts, x1, sizeof(double) * 2 * n1, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(R->d_pts + 2 * n1, x2, sizeof(double) * 2 * n2, cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(R->d_leaves, R->leaves.data(), sizeof(RLeaf) * R->leaves.size(), cudaMemcpyHostToDevice, st);
  for (const auto& lf : R->leaves)
    launch_eval_dense(R->d_pts + 2 * lf.row0, (int)lf.m1, R->d_pts + 2 * (n1 + lf.col0), (int)lf.m2, R->kp, -1,
                      R->d_leafK + lf.off, (int)lf.m1, st);
  if (nb > 0) {
    cudaMemcpyAsync(R->d_blk, R->blk.data(), sizeof(AcaBlock) * nb, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(R->d_status, 0, sizeof(int) * nb, st);
    launch_aca(R->d_pts, R->kp, R->d_blk, nb, maxcap, R->d_panels, R->d_flags, R->d_piv, tol, R->d_rank,
               R->d_status, st);
    for (int q = 0; q < nb; ++q) {
      if (!R->blk[q].grid) continue;
      if (!launch_aca_grid(R->d_pts, R->kp, R->d_blk, q, R->blk[q].cap, R->d_panels, R->d_flags, R->d_piv, tol,
                           R->d_rank, R->d_status, R->d_scr, st))
        launch_aca_one(R->d_pts, R->kp, R->d_blk, q, maxcap, R->d_panels, R->d_flags, R->d_piv, tol, R->d_rank,
                       R->d_status, st);
    }
  }
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    destroy(R);
    return bad(KM_ERR_CUDA, std::string("RKernelHODLR assembly: ") + cudaGetErrorString(e));
  }
  R->rank.assign(nb, 0);
  std::vector<int> stat(nb, 0);
  if (nb > 0) {
    cudaMemcpy(R->rank.data(), R->d_rank, sizeof(int) * nb, cudaMemcpyDeviceToHost);
    cudaMemcpy(stat.data(), R->d_status, sizeof(int) * nb, cudaMemcpyDeviceToHost);
  }
  for (int q = 0; q < nb; ++q) {
    int code = KM_OK;
    std::string msg;
    if (stat[q] == 1) {
      code = KM_ERR_ACA;
      msg = "Incompatible maxrank or matrix dimensions.";
    } else if (stat[q] == 3) {
      code = KM_ERR_TIMEOUT;
      msg = "a bounded grid barrier of the ACA kernel ran out";
    } else if (stat[q] == 2) {
      code = KM_ERR_UNSUPPORTED;
      msg = "ACA rank reached the panel capacity (" + std::to_string(capmax) + " columns) before the tolerance";
    }
    if (code != KM_OK) {
      destroy(R);
      return bad(code, msg);
    }
  }
  // product plan: per depth, block ids and row chunks of V and U
  R->ids_at.assign(std::max(R->levels, 1), {});
  R->vch_at.assign(std::max(R->levels, 1), {});
  R->uch_at.assign(std::max(R->levels, 1), {});
  std::vector<RBlockDev> bdev(nb);
  int64_t part = 0, tslot = 0;
  for (int q = 0; q < nb; ++q) {
    const AcaBlock& b = R->blk[q];
    RBlockDev& B = bdev[q];
    B.row0 = b.row0;
    B.nro = b.nro;
    B.col0 = b.col0 - n1;
    B.ncl = b.ncl;
    B.offU = b.offU;
    B.offV = b.offV;
    B.rank = R->rank[q];
    R->maxrank_seen = std::max(R->maxrank_seen, B.rank);
    B.t = tslot;
    tslot += B.rank;
    B.nchv = (int)((b.ncl + kRectChunk - 1) / kRectChunk);
    B.part0 = part;
    if (B.rank == 0) continue;
    const int d = R->depth[q];
    R->ids_at[d].push_back(q);
    for (int h = 0; h < B.nchv; ++h) {
      const int64_t i0 = (int64_t)h * kRectChunk;
      R->vch_at[d].push_back(RChunk{q, i0, std::min<int64_t>(kRectChunk, b.ncl - i0)});
    }
    for (int64_t i0 = 0; i0 < b.nro; i0 += kRectChunk)
      R->uch_at[d].push_back(RChunk{q, i0, std::min<int64_t>(kRectChunk, b.nro - i0)});
    part += (int64_t)B.nchv * B.rank;
  }
  R->nparts = part;
  R->nt = tslot;
  if (nb > 0 && !ralloc(R, &R->d_bdev, nb)) {
    g_create_error = R->err;
    destroy(R);
    return KM_ERR_OOM;
  }
  if (nb > 0) cudaMemcpy(R->d_bdev, bdev.data(), sizeof(RBlockDev) * nb, cudaMemcpyHostToDevice);
  const int D = std::max(R->levels, 1);
  R->d_ids.assign(D, nullptr);
  R->d_vch.assign(D, nullptr);
  R->d_uch.assign(D, nullptr);
  for (int d = 0; d < D; ++d) {
    if (R->ids_at[d].empty()) continue;
    if (!ralloc(R, &R->d_ids[d], (int64_t)R->ids_at[d].size()) ||
        !ralloc(R, &R->d_vch[d], (int64_t)R->vch_at[d].size()) ||
        !ralloc(R, &R->d_uch[d], (int64_t)R->uch_at[d].size())) {
      g_create_error = R->err;
      destroy(R);
      return KM_ERR_OOM;
    }
    cudaMemcpy(R->d_ids[d], R->ids_at[d].data(), sizeof(int) * R->ids_at[d].size(), cudaMemcpyHostToDevice);
    cudaMemcpy(R->d_vch[d], R->vch_at[d].data(), sizeof(RChunk) * R->vch_at[d].size(), cudaMemcpyHostToDevice);
    cudaMemcpy(R->d_uch[d], R->uch_at[d].data(), sizeof(RChunk) * R->uch_at[d].size(), cudaMemcpyHostToDevice);
  }
  // release the ACA work arrays that the products do not need
  rfree(R, R->d_flags);
  rfree(R, R->d_scr);
  R->d_flags = nullptr;
  R->d_scr = nullptr;
  *out = R;
  return KM_OK;
}

extern "C" int km_rhodlr_destroy(km_rhodlr* R) {
  destroy(R);
  return KM_OK;
}

extern "C" int km_rhodlr_info(const km_rhodlr* R, int64_t* nblocks, int64_t* nleaves, int64_t* levels) {
  if (!R) return KM_ERR_BAD_ARG;
  if (nblocks) *nblocks = (int64_t)R->blk.size();
  if (nleaves) *nleaves = (int64_t)R->leaves.size();
  if (levels) *levels = R->levels;
  return KM_OK;
}

extern "C" int km_rhodlr_block_ranks(const km_rhodlr* R, int64_t* ranks) {
  if (!R || !ranks) return KM_ERR_BAD_ARG;
  for (size_t q = 0; q < R->rank.size(); ++q) ranks[q] = R->rank[q];
  return KM_OK;
}

extern "C" int km_rhodlr_aca_pivots(km_rhodlr* R, int64_t block, int64_t cap, int64_t* rows, int64_t* cols,
                                    int64_t* out_rank) {
  if (!R || !rows || !cols || !out_rank) return KM_ERR_BAD_ARG;
  if (block < 0 || block >= (int64_t)R->blk.size()) return rfail(R, KM_ERR_BAD_ARG, "block out of range");
  cudaSetDevice(R->cfg.device);
  const AcaBlock& b = R->blk[block];
  const int rq = R->rank[block];
  std::vector<int> p(2 * (size_t)b.cap);
  if (cudaMemcpy(p.data(), R->d_piv + 2 * b.offPiv, sizeof(int) * 2 * b.cap, cudaMemcpyDeviceToHost) != cudaSuccess)
    return rfail(R, KM_ERR_CUDA, "pivot copy failed");
  for (int64_t i = 0; i < std::min<int64_t>(cap, rq); ++i) {
    rows[i] = p[i];
    cols[i] = p[b.cap + i];
  }
  *out_rank = rq;
  return KM_OK;
}

extern "C" int km_rhodlr_matvec(km_rhodlr* R, const double* x, double* y, int64_t k) {
  if (!R || !x || !y || k < 1 || k > 65535) return R ? rfail(R, KM_ERR_BAD_ARG, "bad product arguments") : KM_ERR_BAD_ARG;
  cudaSetDevice(R->cfg.device);
  if (!ensure_k(R, k)) return KM_ERR_OOM;
  cudaStream_t st = R->st;
  const int64_t n1 = R->n1, n2 = R->n2;
  cudaMemcpyAsync(R->d_X, x, sizeof(double) * n2 * k, cudaMemcpyHostToDevice, st);
  k_rleaf_apply<<<dim3((unsigned)R->leaves.size(), (unsigned)k), 256, 0, st>>>(R->d_leaves, R->d_leafK, R->d_X, n2,
                                                                             R->d_Y, n1);
  const size_t usm = (size_t)std::max(R->maxrank_seen, 1) * sizeof(double);
  smem_limit((const void*)k_rblock_u, usm);
  for (int d = 0; d < (int)R->ids_at.size(); ++d) {
    if (R->ids_at[d].empty()) continue;
    k_rblock_vt<<<dim3((unsigned)R->vch_at[d].size(), (unsigned)k), 256, 0, st>>>(R->d_vch[d], R->d_bdev,
                                                                                R->d_panels, R->d_X, n2, R->d_part,
                                                                                (int)k);
    k_rblock_tsum<<<dim3((unsigned)R->ids_at[d].size(), (unsigned)k), 128, 0, st>>>(R->d_ids[d], R->d_bdev,
                                                                                   R->d_part, R->d_T, (int)k);
    k_rblock_u<<<dim3((unsigned)R->uch_at[d].size(), (unsigned)k), 256, usm, st>>>(R->d_uch[d], R->d_bdev,
                                                                                  R->d_panels, R->d_T, R->d_Y, n1,
                                                                                  (int)k);
  }
  cudaMemcpyAsync(y, R->d_Y, sizeof(double) * n1 * k, cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return rfail(R, KM_ERR_CUDA, std::string("RKernelHODLR product: ") + cudaGetErrorString(e));
  return KM_OK;
}
