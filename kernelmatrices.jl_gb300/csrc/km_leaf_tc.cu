// Mixed-precision leaf stage on the tensor cores: blocked Cholesky of the augmented leaf matrix
//
//     [ K_j     ]   =   [ L_j ] [ L_j' A_j ]        A_j = L_j^{-1} Phi_j
//     [ Phi_j'  ]       [ A_j']
//
// so that one factorisation gives the leaf factor L_j (leaf Cholesky, src/HODLR/src/symfact.jl:17)
// and the transformed leaf panel A_j = L_j^{-1} Phi_j (the leaf-level invapply!,
// src/HODLR/src/utils.jl:54-65, BlockDiagonal.jl:62-66) in float pairs.  The rows of Phi_j' are
// the columns of A_j as stored (m x r column-major), so "row g" of the lower part is column g of
// the panel buffer.
//
// Per 64-column block (step) of every leaf:
//   * k_lc_panel (CUDA cores, one CTA per leaf): Cholesky of the 64 x 64 diagonal block, then
//     the block column below it by forward substitution x D' = a per row (float pairs, Dot2
//     sums), written back, and every row of the block column cut into kSlices bf16 slices with
//     a row exponent (km_tc.cuh) in the tensor cores' shared-memory layout;
//   * k_lc_update (tensor cores, one CTA per 128 x 64 tile of the trailing rows / columns):
//     C -= P P' from the slices: the 28 slice products with i + j <= 6 accumulate per diagonal
//     i + j in tensor memory (exact integer sums in fp32), and the epilogue adds the 7 diagonal
//     sums in float pairs, scales by 2^(e_row + e_col) and subtracts from C.
// The first step reads the FP64 leaf matrix K_j directly (conversion to float pairs on load).
#include "km_kernels.h"
#include "km_tc.cuh"

namespace km {

using tc::kSlices;

constexpr int kLcNB = 64;            // panel width = K of the update products
constexpr int kLcTileM = 128;        // rows of an update tile (MMA M)
constexpr int kLcTileN = 64;         // columns of an update tile (MMA N)
constexpr int kLcPanelThreads = 128;
constexpr int kLcUpdThreads = 256;   // 8 warps: warp w reads tensor-memory lanes 32 (w % 4) ..
constexpr uint32_t kLcTmemCols = 512;  // kSlices x kLcTileN = 448 accumulator columns
constexpr uint32_t kATileBytes = kLcTileM * kLcNB * 2;  // one slice of a 128-row tile
constexpr uint32_t kBTileBytes = kLcTileN * kLcNB * 2;  // one slice of a 64-row tile
constexpr long long kTcWaitLimit = 1ll << 21;           // mbarrier polls before giving up
constexpr int kLcMaxLeaf = 1024;
constexpr int kLcMaxRank = 256;

__host__ __device__ inline int64_t lc_rows_padded(int64_t rows) { return (rows + 127) / 128 * 128; }

// bf16 element index of (slice s, row rho, column c) in the slice array of one leaf and step:
// core matrix (rho / 8, c / 8) of slice s is 64 consecutive elements, core matrices ordered by
// slice, then row group, then column group; rp = padded rows of the step.
__host__ __device__ inline int64_t lc_slice_index(int s, int64_t rp, int64_t rho, int c) {
  return ((((int64_t)s * (rp / 8) + rho / 8) * 8 + c / 8) * 64) + (rho % 8) * 8 + (c % 8);
}

// Writes the kSlices slices of 8 consecutive values (columns 8 kc .. 8 kc + 7 of row rho).
__device__ __forceinline__ void store_slices8(uint16_t* base, int64_t rp, int64_t rho, int kc, const ff (&x)[8],
                                              int e) {
  uint32_t w[kSlices][4];
#pragma unroll
  for (int cc = 0; cc < 8; cc += 2) {
    float t0[kSlices], t1[kSlices];
    tc::split_slices(x[cc], e, t0);
    tc::split_slices(x[cc + 1], e, t1);
#pragma unroll
    for (int s = 0; s < kSlices; ++s) w[s][cc / 2] = tc::bf16_pack2(t0[s], t1[s]);
  }
#pragma unroll
  for (int s = 0; s < kSlices; ++s)
    *reinterpret_cast<uint4*>(base + lc_slice_index(s, rp, rho, 8 * kc)) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
}

// ---------------------------------------------------------------------------------------------
// Panel step: grid = nleaf, block = kLcPanelThreads.
// ---------------------------------------------------------------------------------------------
template <bool FROM_K>
__global__ void __launch_bounds__(kLcPanelThreads) k_lc_panel(const double* __restrict__ K, ff* __restrict__ Lf,
                                                              ff* __restrict__ G, int r, DTree t, int c0,
                                                              uint16_t* __restrict__ slices, int* __restrict__ rexp,
                                                              int64_t slice_stride, int64_t exp_stride,
                                                              int* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char lc_smem_p[];
  constexpr int LD = kLcNB + 1;
  ff* D = reinterpret_cast<ff*>(lc_smem_p);  // kLcNB x LD, D[i * LD + c]
  ff* xs = D + kLcNB * LD;               // kLcNB x NT, xs[c * NT + tid]
  __shared__ ff dinv[kLcNB];
  __shared__ int sbad;
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  if (c0 >= m) return;
  const int nb = min(kLcNB, m - c0);
  const int64_t koff = d_leaf_koff(t, leaf);
  const int64_t qoff = d_leaf_start(t, leaf) * r;
  const int T = m - c0 - nb;  // trailing rows of K_j
  const int R = T + r;        // rows below the block: trailing K rows, then the r rows of Phi'
  const int64_t RP = lc_rows_padded(R);
  uint16_t* sl = slices + leaf * slice_stride;
  int* ex = rexp + leaf * exp_stride;
  const int tid = threadIdx.x, NT = blockDim.x;
  auto src = [&](int row, int col) -> ff {  // lower-triangle entry of the matrix being factored
    const int64_t o = koff + (int64_t)col * m + row;
    if (FROM_K) return ff(K[o]);
    return Lf[o];
  };
  // (1) diagonal block: unblocked Cholesky in shared memory
  for (int e = tid; e < nb * nb; e += NT) {
    const int i = e % nb, c = e / nb;
    if (i >= c) D[i * LD + c] = src(c0 + i, c0 + c);
  }
  if (tid == 0) sbad = 0;
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    const ff d = D[j * LD + j];
    const bool ok = d > 0.0;
    const ff sd = ok ? sqrt(d) : ff(1.0);
    if (!ok && tid == 0 && sbad == 0) sbad = c0 + j + 1;
    __syncthreads();
    for (int i = j + 1 + tid; i < nb; i += NT) D[i * LD + j] /= sd;
    if (tid == 0) D[j * LD + j] = sd;
    __syncthreads();
    const int w = nb - j - 1;
    for (int e = tid; e < w * w; e += NT) {
      const int i = j + 1 + e % w, c = j + 1 + e / w;
      if (i >= c) D[i * LD + c] -= D[i * LD + j] * D[c * LD + j];
    }
    __syncthreads();
  }
  for (int c = tid; c < nb; c += NT) dinv[c] = ff(1.0) / D[c * LD + c];
  for (int e = tid; e < nb * nb; e += NT) {
    const int i = e % nb, c = e / nb;
    if (i >= c) Lf[koff + (int64_t)(c0 + c) * m + c0 + i] = D[i * LD + c];
  }
  if (tid == 0 && sbad != 0 && info[leaf] == 0) info[leaf] = sbad;
  __syncthreads();
  // (2) rows below: x D' = a, one row per thread; then the row's slices
  for (int64_t base = 0; base < RP; base += NT) {
    const int64_t rho = base + tid;
    const bool valid = rho < R;
    float amax = 0.f;
    if (valid) {
      for (int c = 0; c < nb; ++c) {
        const ff a = rho < T ? src(c0 + nb + (int)rho, c0 + c) : G[qoff + (rho - T) * m + c0 + c];
        acc_t<ff> acc(a);
        for (int k = 0; k < c; ++k) acc -= xs[k * NT + tid] * D[c * LD + k];
        const ff x = accv(acc) * dinv[c];
        xs[c * NT + tid] = x;
        amax = fmaxf(amax, fabsf(x.hi));
      }
      for (int c = 0; c < nb; ++c) {
        const ff x = xs[c * NT + tid];
        if (rho < T)
          Lf[koff + (int64_t)(c0 + c) * m + c0 + nb + rho] = x;
        else
          G[qoff + (rho - T) * m + c0 + c] = x;
      }
    }
    const int e = tc::row_exponent(amax);
    ex[rho] = e;
#pragma unroll 1
    for (int kc = 0; kc < kLcNB / 8; ++kc) {
      ff x[8];
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) {
        const int c = 8 * kc + cc;
        x[cc] = (valid && c < nb) ? xs[c * NT + tid] : ff(0.0);
      }
      store_slices8(sl, RP, rho, kc, x, e);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Trailing update step: grid = (nleaf, row tiles, column tiles), block = kLcUpdThreads.
// Shared memory: kSlices A slices (kATileBytes each), then kSlices B slices (kBTileBytes each).
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void lc_issue_products(uint32_t tmem, uint32_t smA, uint32_t smB) {
  constexpr uint32_t idesc = tc::idesc_bf16(kLcTileM, kLcTileN);
#pragma unroll 1
  for (int d = 0; d < kSlices; ++d) {
    bool first = true;
#pragma unroll 1
    for (int i = 0; i <= d; ++i) {
      const int j = d - i;
#pragma unroll
      for (int ks = 0; ks < kLcNB / 16; ++ks) {
        const uint64_t ad = tc::smem_desc(smA + i * kATileBytes + ks * 256, 128, 1024);
        const uint64_t bd = tc::smem_desc(smB + j * kBTileBytes + ks * 256, 128, 1024);
        tc::mma_bf16(tmem + d * kLcTileN, ad, bd, idesc, !first);
        first = false;
      }
    }
  }
}

template <bool FROM_K>
__global__ void __launch_bounds__(kLcUpdThreads, 1) k_lc_update(const double* __restrict__ K, ff* __restrict__ Lf,
                                                                ff* __restrict__ G, int r, DTree t, int c0,
                                                                const uint16_t* __restrict__ slices,
                                                                const int* __restrict__ rexp, int64_t slice_stride,
                                                                int64_t exp_stride, int* __restrict__ info) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tslot;
  __shared__ int cexp[kLcTileN];
  __shared__ int serr;
  const int64_t leaf = blockIdx.x;
  const int rt = blockIdx.y, ct = blockIdx.z;
  const int m = d_leaf_size(t, leaf);
  if (c0 >= m) return;
  const int nb = min(kLcNB, m - c0);
  const int T = m - c0 - nb;
  const int R = T + r;
  if (T <= 0 || kLcTileM * rt >= R || kLcTileN * ct >= T) return;
  const int rlast = min(kLcTileM * rt + kLcTileM - 1, R - 1);
  if (rlast < T && rlast < kLcTileN * ct) return;  // tile strictly above the diagonal
  const int64_t RP = lc_rows_padded(R);
  const int64_t koff = d_leaf_koff(t, leaf);
  const int64_t qoff = d_leaf_start(t, leaf) * r;
  const uint16_t* sl = slices + leaf * slice_stride;
  const int* ex = rexp + leaf * exp_stride;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const uint32_t smA = tc::smem_u32(smraw);
  const uint32_t smB = smA + kSlices * kATileBytes;

  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::mbar_fence_init();
    serr = 0;
  }
  if (w == 0) {
    tc::tmem_alloc(&tslot, kLcTmemCols);
    tc::tmem_relinquish();
  }
  if (tid < kLcTileN) {
    const int64_t j = (int64_t)kLcTileN * ct + tid;
    cexp[tid] = j < RP ? ex[j] : 0;
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tslot;

  if (tid == 0) {
    tc::mbar_arrive_expect_tx(&bar[0], kSlices * (kATileBytes + kBTileBytes));
    for (int s = 0; s < kSlices; ++s) {
      tc::bulk_g2s(smraw + s * kATileBytes, sl + lc_slice_index(s, RP, (int64_t)kLcTileM * rt, 0), kATileBytes,
                   &bar[0]);
      tc::bulk_g2s(smraw + kSlices * kATileBytes + s * kBTileBytes,
                   sl + lc_slice_index(s, RP, (int64_t)kLcTileN * ct, 0), kBTileBytes, &bar[0]);
    }
    if (tc::mbar_wait(&bar[0], 0, kTcWaitLimit)) {
      tc::tc_fence_after();
      lc_issue_products(tmem, smA, smB);
    } else {
      serr = 1;
    }
    tc::mma_commit(&bar[1]);
  }
  __syncwarp();
  const bool done = tc::mbar_wait(&bar[1], 0, kTcWaitLimit);
  tc::tc_fence_after();
  __syncthreads();
  if (!done || serr) {
    if (tid == 0) {
      tc::mbar_wait(&bar[0], 0, kTcWaitLimit);  // copies still in flight land before the exit
      info[leaf] = -1;
    }
  } else {
    // epilogue: warp w reads lanes 32 (w % 4) + lane = tile row, columns 32 (w / 4) .. + 31
    const int q = w & 3, h = w >> 2;
    const int64_t rho = (int64_t)kLcTileM * rt + 32 * q + lane;
    const bool rvalid = rho < R;
    const int erow = rvalid ? ex[rho] : 0;
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
#pragma unroll 1
    for (int cc = 0; cc < 4; ++cc) {
      const int j0 = 32 * h + 8 * cc;
      float s[kSlices][8];
#pragma unroll
      for (int d = 0; d < kSlices; ++d) tc::tmem_ld8(tl + d * kLcTileN + j0, s[d]);
      tc::tmem_wait_ld();
      if (!rvalid) continue;
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        const int j = kLcTileN * ct + j0 + jj;  // trailing column
        if (j >= T || (rho < T && rho < j)) continue;
        float sd[kSlices];
#pragma unroll
        for (int d = 0; d < kSlices; ++d) sd[d] = s[d][jj];
        const ff v = tc::ff_ldexp(tc::combine_diagonals(sd), erow + cexp[j0 + jj]);
        if (rho < T) {
          const int64_t o = koff + (int64_t)(c0 + nb + j) * m + c0 + nb + rho;
          const ff cv = FROM_K ? ff(K[o]) : Lf[o];
          Lf[o] = cv - v;
        } else {
          const int64_t o = qoff + (rho - T) * m + c0 + nb + j;
          G[o] = G[o] - v;
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (w == 0) tc::tmem_dealloc(tmem, kLcTmemCols);
}

// ---------------------------------------------------------------------------------------------
// Probe of the split product (C ABI: km_probe_tc_gemm): C = A B' for A 128 x 64 and B 64 x 64
// (row-major doubles).  mode 0: A and B hold integers |v| <= 128, used as the single slice;
// C is the tensor cores' fp32 sum.  mode 1: the float-pair split product of arbitrary values.
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kLcUpdThreads, 1) k_tc_probe(const double* __restrict__ A,
                                                               const double* __restrict__ B, int mode,
                                                               double* __restrict__ C, int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ int rexp[kLcTileM + kLcTileN];
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  uint16_t* sA = reinterpret_cast<uint16_t*>(smraw);
  uint16_t* sB = sA + kSlices * kATileBytes / 2;
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
  }
  if (w == 0) {
    tc::tmem_alloc(&tslot, kLcTmemCols);
    tc::tmem_relinquish();
  }
  if (tid < kLcTileM + kLcTileN) {
    const bool isA = tid < kLcTileM;
    const int row = isA ? tid : tid - kLcTileM;
    const double* src = isA ? A + row * kLcNB : B + row * kLcNB;
    uint16_t* dst = isA ? sA : sB;
    const int64_t rp = isA ? kLcTileM : kLcTileN;
    float amax = 0.f;
    for (int c = 0; c < kLcNB; ++c) amax = fmaxf(amax, fabsf((float)src[c]));
    const int e = mode == 0 ? 7 : tc::row_exponent(amax);  // mode 0: v = t 2^-7 2^7 = t
    rexp[tid] = e;
    for (int kc = 0; kc < kLcNB / 8; ++kc) {
      ff x[8];
      for (int cc = 0; cc < 8; ++cc) x[cc] = ff(src[8 * kc + cc]);
      store_slices8(dst, rp, row, kc, x, e);
    }
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tslot;
  const uint32_t smA = tc::smem_u32(sA), smB = tc::smem_u32(sB);
  if (tid == 0) {
    if (mode == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16(kLcTileM, kLcTileN);
      for (int ks = 0; ks < kLcNB / 16; ++ks)
        tc::mma_bf16(tmem, tc::smem_desc(smA + ks * 256, 128, 1024), tc::smem_desc(smB + ks * 256, 128, 1024),
                     idesc, ks > 0);
    } else {
      lc_issue_products(tmem, smA, smB);
    }
    tc::mma_commit(&bar);
  }
  __syncwarp();
  const bool done = tc::mbar_wait(&bar, 0, kTcWaitLimit);
  tc::tc_fence_after();
  __syncthreads();
  if (!done) {
    if (tid == 0) status[0] = 1;
  } else {
    const int q = w & 3, h = w >> 2;
    const int row = 32 * q + lane;
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
    for (int cc = 0; cc < 4; ++cc) {
      const int j0 = 32 * h + 8 * cc;
      float s[kSlices][8];
#pragma unroll
      for (int d = 0; d < kSlices; ++d) tc::tmem_ld8(tl + d * kLcTileN + j0, s[d]);
      tc::tmem_wait_ld();
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        double out;
        if (mode == 0) {
          out = (double)s[0][jj];
        } else {
          float sd[kSlices];
#pragma unroll
          for (int d = 0; d < kSlices; ++d) sd[d] = s[d][jj];
          out = (double)tc::ff_ldexp(tc::combine_diagonals(sd), rexp[row] + rexp[kLcTileM + j0 + jj]);
        }
        C[row * kLcTileN + j0 + jj] = out;
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (w == 0) tc::tmem_dealloc(tmem, kLcTmemCols);
}

// ---------------------------------------------------------------------------------------------
// launchers: step p covers columns [64 p, 64 p + 64) of every leaf; the update of step p exists
// when some leaf has rows left after the block
// ---------------------------------------------------------------------------------------------
static int64_t lc_rp_max(const Tree& t, int r) { return lc_rows_padded(t.max_leaf + r); }

bool leaf_chol_tc_supported(const Tree& t, int r) {
  return t.max_leaf >= 1 && t.max_leaf <= kLcMaxLeaf && r >= 1 && r <= kLcMaxRank;
}

int64_t leaf_chol_tc_scratch_bytes(const Tree& t, int r) {
  const int64_t rp = lc_rp_max(t, r);
  return t.nleaf * (rp * kLcNB * kSlices * (int64_t)sizeof(uint16_t) + rp * (int64_t)sizeof(int));
}

int leaf_chol_tc_steps(const Tree& t) { return (int)((t.max_leaf + kLcNB - 1) / kLcNB); }

bool leaf_chol_tc_has_update(const Tree& t, int p) { return t.max_leaf - (int64_t)kLcNB * (p + 1) > 0; }

struct LcArgs {
  uint16_t* slices;
  int* rexp;
  int64_t slice_stride, exp_stride;
};

static LcArgs lc_args(const Tree& t, int r, void* scratch) {
  const int64_t rp = lc_rp_max(t, r);
  LcArgs a;
  a.slice_stride = rp * kLcNB * kSlices;
  a.exp_stride = rp;
  a.slices = reinterpret_cast<uint16_t*>(scratch);
  a.rexp = reinterpret_cast<int*>(a.slices + t.nleaf * a.slice_stride);
  return a;
}

void launch_leaf_chol_tc_panel(const double* K, ff* Lf, ff* G, int r, const Tree& t, int p, void* scratch,
                               int* info, cudaStream_t st) {
  const LcArgs a = lc_args(t, r, scratch);
  const size_t smp = (size_t)kLcNB * (kLcNB + 1) * sizeof(ff) + (size_t)kLcNB * kLcPanelThreads * sizeof(ff);
  const int c0 = kLcNB * p;
  if (p == 0) {
    smem_limit((const void*)k_lc_panel<true>, smp);
    k_lc_panel<true><<<(unsigned)t.nleaf, kLcPanelThreads, smp, st>>>(K, Lf, G, r, dtree(t), c0, a.slices, a.rexp,
                                                                      a.slice_stride, a.exp_stride, info);
  } else {
    smem_limit((const void*)k_lc_panel<false>, smp);
    k_lc_panel<false><<<(unsigned)t.nleaf, kLcPanelThreads, smp, st>>>(K, Lf, G, r, dtree(t), c0, a.slices, a.rexp,
                                                                       a.slice_stride, a.exp_stride, info);
  }
}

void launch_leaf_chol_tc_update(const double* K, ff* Lf, ff* G, int r, const Tree& t, int p, void* scratch,
                                int* info, cudaStream_t st) {
  const LcArgs a = lc_args(t, r, scratch);
  const size_t smu = (size_t)kSlices * (kATileBytes + kBTileBytes);
  const int c0 = kLcNB * p;
  const int64_t tmax = t.max_leaf - c0 - kLcNB;
  if (tmax <= 0) return;
  dim3 grid((unsigned)t.nleaf, (unsigned)((tmax + r + kLcTileM - 1) / kLcTileM),
            (unsigned)((tmax + kLcTileN - 1) / kLcTileN));
  if (p == 0) {
    smem_limit((const void*)k_lc_update<true>, smu);
    k_lc_update<true><<<grid, kLcUpdThreads, smu, st>>>(K, Lf, G, r, dtree(t), c0, a.slices, a.rexp, a.slice_stride,
                                                        a.exp_stride, info);
  } else {
    smem_limit((const void*)k_lc_update<false>, smu);
    k_lc_update<false><<<grid, kLcUpdThreads, smu, st>>>(K, Lf, G, r, dtree(t), c0, a.slices, a.rexp,
                                                         a.slice_stride, a.exp_stride, info);
  }
}

}  // namespace km

extern "C" int km_probe_tc_gemm(int device, const double* A, const double* B, int mode, double* C) {
  using namespace km;
  if (!A || !B || !C || (mode != 0 && mode != 1)) return KM_ERR_BAD_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return KM_ERR_CUDA;
  double *dA = nullptr, *dB = nullptr, *dC = nullptr;
  int* dst = nullptr;
  const size_t na = (size_t)kLcTileM * kLcNB, nbb = (size_t)kLcTileN * kLcNB, nc = (size_t)kLcTileM * kLcTileN;
  int rc = KM_OK;
  if (cudaMalloc(&dA, na * 8) != cudaSuccess || cudaMalloc(&dB, nbb * 8) != cudaSuccess ||
      cudaMalloc(&dC, nc * 8) != cudaSuccess || cudaMalloc(&dst, sizeof(int)) != cudaSuccess) {
    rc = KM_ERR_OOM;
  } else {
    cudaMemcpy(dA, A, na * 8, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B, nbb * 8, cudaMemcpyHostToDevice);
    cudaMemset(dst, 0, sizeof(int));
    const size_t smu = (size_t)kSlices * (kATileBytes + kBTileBytes);
    smem_limit((const void*)k_tc_probe, smu);
    k_tc_probe<<<1, kLcUpdThreads, smu>>>(dA, dB, mode, dC, dst);
    int stv = 0;
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
      rc = KM_ERR_CUDA;
    } else {
      cudaMemcpy(&stv, dst, sizeof(int), cudaMemcpyDeviceToHost);
      cudaMemcpy(C, dC, nc * 8, cudaMemcpyDeviceToHost);
      if (stv) rc = KM_ERR_TIMEOUT;
    }
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(dst);
  return rc;
}
