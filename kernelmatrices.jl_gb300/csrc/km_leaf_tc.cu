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
//   * k_lc_diag (CUDA cores, one CTA per leaf): Cholesky D of the 64 x 64 diagonal block and,
//     in the same column sweep, X = D^{-1} (float pairs, shared memory); the rows of X cut into
//     bf16 slices for the next kernel;
//   * k_lc_trsm (tensor cores, one CTA per 128-row tile of the rows below the block: trailing
//     rows of K_j, then the rows of Phi_j'): the block column P = A X' (the triangular solve
//     P D' = A with the explicit inverse of the diagonal block) as a split product, written back
//     and cut into slices (with row exponents) for the update;
//   * k_lc_update (tensor cores, one CTA per 128 x 64 tile of the trailing rows / columns):
//     C -= P P' from the slices.
// A float-pair value is cut into kSlices bf16 slices with a row exponent (km_tc.cuh); both
// products take the 28 slice products with i + j <= 6, accumulated per diagonal i + j in tensor
// memory (exact integer sums in fp32), and the epilogues add the 7 diagonal sums in float pairs
// and scale them by 2^(e_row + e_col).  The leaf matrices enter in float pairs (written by the
// mixed-form leaf evaluation).
#include "km_kernels.h"
#include "km_tc.cuh"

namespace km {

using tc::kSlices;

constexpr int kLcNB = 64;              // panel width = K of the products
constexpr int kLcTileM = 128;          // rows of a tile (MMA M)
constexpr int kLcTileN = 64;           // columns of a tile (MMA N)
constexpr int kLcTcThreads = 512;      // 16 warps: warp w reads tensor-memory lanes 32 (w % 4) .. + 31,
                                       // columns 16 (w / 4) .. + 15 of a tile
constexpr int kLcDiagThreads = 512;
constexpr int kLcDiagCols = kLcNB * kLcNB / kLcDiagThreads;  // trailing-update columns a thread
constexpr int kLcProbeThreads = 256;
constexpr uint32_t kLcTmemCols = 512;  // kSlices x kLcTileN = 448 accumulator columns
constexpr uint32_t kATileBytes = kLcTileM * kLcNB * 2;  // one slice of a 128-row tile
constexpr uint32_t kBTileBytes = kLcTileN * kLcNB * 2;  // one slice of a 64-row tile
constexpr long long kTcWaitLimit = 1ll << 21;           // mbarrier polls before giving up
constexpr int kLcMaxLeaf = 1024;
constexpr int kLcMaxRank = 256;

__host__ __device__ inline int64_t lc_rows_padded(int64_t rows) { return (rows + 127) / 128 * 128; }

// bf16 element index of (slice s, row rho, column c) in a slice array of rp rows: core matrix
// (rho / 8, c / 8) of slice s is 64 consecutive elements, core matrices ordered by slice, then
// row group, then column group.
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
    *reinterpret_cast<uint4*>(base + lc_slice_index(s, rp, rho, 8 * kc)) =
        make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
}

// Split products of one 128 x 64 tile: A slices (kSlices x kATileBytes) times B slices
// (kSlices x kBTileBytes) into kSlices accumulators of kLcTileN columns, one per diagonal i + j.
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

// The 8 float-pair values of accumulator columns j0 .. j0 + 7 of this thread's lane: the 7
// diagonal sums combined and scaled by 2^(erow + ecol[jj]).
__device__ __forceinline__ void lc_tile_values(uint32_t tl, int j0, int erow, const int* ecol, ff (&out)[8]) {
  float s[kSlices][8];
#pragma unroll
  for (int d = 0; d < kSlices; ++d) tc::tmem_ld8(tl + d * kLcTileN + j0, s[d]);
  tc::tmem_wait_ld();
#pragma unroll
  for (int jj = 0; jj < 8; ++jj) {
    float sd[kSlices];
#pragma unroll
    for (int d = 0; d < kSlices; ++d) sd[d] = s[d][jj];
    out[jj] = tc::ff_ldexp(tc::combine_diagonals(sd), erow + ecol[jj]);
  }
}

// ---------------------------------------------------------------------------------------------
// Diagonal block: grid = nleaf, block = kLcDiagThreads, dynamic shared memory 2 x 64 x 65 float
// pairs.  D = chol(B) and X = D^{-1} for the block B = rows / columns [c0, c0 + nb) of the
// matrix being factored (row j of X is finalised at step j, then rows i > j subtract L_ij X_j);
// beyond nb both are the identity.  Writes D to Lf and the slices of the rows of X (64 rows,
// the canonical layout) with their exponents.
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kLcDiagThreads) k_lc_diag(ff* __restrict__ Lf, DTree t, int c0,
                                                            uint16_t* __restrict__ xsl, int* __restrict__ xexp,
                                                            int* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char lc_smem_d[];
  constexpr int LD = kLcNB + 1;
  ff* D = reinterpret_cast<ff*>(lc_smem_d);
  ff* X = D + kLcNB * LD;
  __shared__ int sbad;
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  if (c0 >= m) return;
  const int nb = min(kLcNB, m - c0);
  const int64_t koff = d_leaf_koff(t, leaf);
  const int tid = threadIdx.x, NT = blockDim.x;
  for (int e = tid; e < kLcNB * kLcNB; e += NT) {
    const int i = e % kLcNB, c = e / kLcNB;
    ff v(0.0);
    if (i < nb && c < nb) {
      if (i >= c) v = Lf[koff + (int64_t)(c0 + c) * m + c0 + i];
    } else if (i == c) {
      v = ff(1.0);
    }
    D[i * LD + c] = v;
    X[i * LD + c] = ff(i == c ? 1.0 : 0.0);
  }
  if (tid == 0) sbad = 0;
  __syncthreads();
  // two barriers a column: every thread forms the pivot from D[j][j] (left in place until the
  // end, the factor's diagonal goes to sdiag) and scales its share of column j and of row j of X;
  // then the trailing update
  __shared__ ff sdiag[kLcNB];
  for (int j = 0; j < nb; ++j) {
    const ff d = D[j * LD + j];
    const bool ok = d > 0.0;
    const ff sd = ok ? sqrt(d) : ff(1.0);
    const ff rinv = ff(1.0) / sd;
    if (!ok && tid == 0 && sbad == 0) sbad = c0 + j + 1;
    for (int i = j + 1 + tid; i < nb; i += NT) D[i * LD + j] = ff(D[i * LD + j] * rinv);
    for (int c = tid; c <= j; c += NT) X[j * LD + c] = ff(X[j * LD + c] * rinv);
    if (tid == 0) sdiag[j] = sd;
    __syncthreads();
    // trailing lower triangle of D (i >= c > j) and rows i > j of X (columns c <= j): thread
    // (row i = tid % 64, columns kLcDiagCols g .. + kLcDiagCols - 1 with g = tid / 64), the row's
    // pivot-column entry loaded once
    for (int e = tid; e < kLcNB * (kLcNB / kLcDiagCols); e += NT) {
      const int i = e & (kLcNB - 1), g = e / kLcNB;
      if (i > j && i < nb) {
        const ff lij = D[i * LD + j];
#pragma unroll
        for (int c = kLcDiagCols * g; c < kLcDiagCols * g + kLcDiagCols; ++c) {
          if (c <= j) X[i * LD + c] -= lij * X[j * LD + c];
          else if (c <= i) D[i * LD + c] -= lij * D[c * LD + j];
        }
      }
    }
    __syncthreads();
  }
  for (int j = tid; j < nb; j += NT) D[j * LD + j] = sdiag[j];
  __syncthreads();
  // L in the lower triangle of the diagonal block; the strictly lower part of X = D^{-1} in its
  // (otherwise unused) strictly upper triangle, X[i][c] at row c0 + c, column c0 + i, for the
  // block solves of k_leaf_tri_blk (X's diagonal is 1 / D_ii, recomputed there the same way)
  for (int e = tid; e < nb * nb; e += NT) {
    const int i = e % nb, c = e / nb;
    if (i >= c) Lf[koff + (int64_t)(c0 + c) * m + c0 + i] = D[i * LD + c];
    else Lf[koff + (int64_t)(c0 + c) * m + c0 + i] = X[c * LD + i];
  }
  if (tid == 0 && sbad != 0 && info[leaf] == 0) info[leaf] = sbad;
  // rows of X: four threads per row, 16 columns each
  uint16_t* dst = xsl + leaf * (int64_t)(kSlices * kLcNB * kLcNB);
  for (int rr = tid >> 2; rr < kLcNB; rr += NT >> 2) {
    const int qq = tid & 3;
    float amax = 0.f;
    ff xv[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      xv[k] = X[rr * LD + 16 * qq + k];
      amax = fmaxf(amax, fabsf(xv[k].hi));
    }
    amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, 1));
    amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, 2));
    const int e = tc::row_exponent(amax);
    if (qq == 0) xexp[leaf * kLcNB + rr] = e;
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      ff xg[8];
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) xg[cc] = xv[8 * g + cc];
      store_slices8(dst, kLcNB, rr, 2 * qq + g, xg, e);
    }
  }
}

// ---------------------------------------------------------------------------------------------
// Block column below the diagonal block: grid = (nleaf, row tiles), block = kLcTcThreads,
// dynamic shared memory kSlices x (kATileBytes + kBTileBytes).  Rows [128 rt, 128 rt + 128) of
// the rows below (trailing rows of K_j, then the r rows of Phi_j', then zero padding up to RP).
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kLcTcThreads, 1) k_lc_trsm(ff* __restrict__ Lf, ff* __restrict__ G, int r,
                                                             DTree t, int c0, const uint16_t* __restrict__ xsl,
                                                             const int* __restrict__ xexp,
                                                             uint16_t* __restrict__ slices, int* __restrict__ rexp,
                                                             int64_t slice_stride, int64_t exp_stride,
                                                             int* __restrict__ info) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  constexpr int LD = kLcNB + 1;
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tslot;
  __shared__ int serr;
  __shared__ int bexp[kLcNB];
  __shared__ int aexp[kLcTileM];
  const int64_t leaf = blockIdx.x;
  const int rt = blockIdx.y;
  const int m = d_leaf_size(t, leaf);
  if (c0 >= m) return;
  const int nb = min(kLcNB, m - c0);
  const int T = m - c0 - nb;
  const int R = T + r;
  const int64_t RP = lc_rows_padded(R);
  if ((int64_t)kLcTileM * rt >= RP) return;
  const int64_t koff = d_leaf_koff(t, leaf);
  const int64_t qoff = d_leaf_start(t, leaf) * r;
  uint16_t* sl = slices + leaf * slice_stride;
  int* ex = rexp + leaf * exp_stride;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  uint16_t* sA = reinterpret_cast<uint16_t*>(smraw);
  uint16_t* sB = sA + kSlices * kATileBytes / 2;
  ff* Pst = reinterpret_cast<ff*>(smraw);  // after the products: P, kLcTileM x LD
  const uint32_t smA = tc::smem_u32(sA), smB = tc::smem_u32(sB);

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
  if (tid < kLcNB) bexp[tid] = xexp[leaf * kLcNB + tid];
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tslot;
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(&bar[0], kSlices * kBTileBytes);
    const uint16_t* xs = xsl + leaf * (int64_t)(kSlices * kLcNB * kLcNB);
    for (int s = 0; s < kSlices; ++s)
      tc::bulk_g2s(reinterpret_cast<unsigned char*>(sB) + s * kBTileBytes, xs + (int64_t)s * kLcNB * kLcNB,
                   kBTileBytes, &bar[0]);
  }
  // A slices: four threads per row, 16 columns each
  const int i4 = tid >> 2, qq = tid & 3;
  const int64_t rho4 = (int64_t)kLcTileM * rt + i4;
  const bool valid4 = rho4 < R;
  {
    ff a[16];
    float amax = 0.f;
#pragma unroll
    for (int cc = 0; cc < 16; ++cc) {
      const int c = 16 * qq + cc;
      ff v(0.0);
      if (valid4 && c < nb)
        v = rho4 < T ? Lf[koff + (int64_t)(c0 + c) * m + c0 + nb + rho4] : G[qoff + (rho4 - T) * m + c0 + c];
      a[cc] = v;
      amax = fmaxf(amax, fabsf(v.hi));
    }
    amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, 1));
    amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, 2));
    const int e = tc::row_exponent(amax);
    if (qq == 0) aexp[i4] = e;
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      ff xg[8];
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) xg[cc] = a[8 * g + cc];
      store_slices8(sA, kLcTileM, i4, 2 * qq + g, xg, e);
    }
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (tid == 0) {
    if (tc::mbar_wait(&bar[0], 0, kTcWaitLimit)) {
      tc::tc_fence_after();
      lc_issue_products(tmem, smA, smB);
    } else {
      serr = 1;
    }
    tc::mma_commit(&bar[1]);
  }
  __syncwarp();
  if (!tc::mbar_wait(&bar[1], 0, kTcWaitLimit)) atomicExch(&serr, 1);
  tc::tc_fence_after();
  __syncthreads();  // serr is the same in every thread from here on
  if (serr) {
    if (tid == 0) {  // copies and products still in flight finish before the exit
      tc::mbar_wait(&bar[0], 0, kTcWaitLimit);
      tc::mbar_wait(&bar[1], 0, kTcWaitLimit);
      info[leaf] = -1;
    }
  } else {
    // P = A X' into shared memory (over the A slices, which the products have read)
    const int q = w & 3, h = w >> 2;
    const int i = 32 * q + lane;
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
#pragma unroll 1
    for (int cc = 0; cc < 2; ++cc) {
      const int j0 = 16 * h + 8 * cc;
      ff pv[8];
      lc_tile_values(tl, j0, aexp[i], bexp + j0, pv);
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) Pst[i * LD + j0 + jj] = pv[jj];
    }
    __syncthreads();
    // P back to Lf / G, its row exponent and slices for the update step
    ff pv[16];
    float amax = 0.f;
#pragma unroll
    for (int cc = 0; cc < 16; ++cc) {
      const int c = 16 * qq + cc;
      const ff v = (valid4 && c < nb) ? Pst[i4 * LD + c] : ff(0.0);
      pv[cc] = v;
      amax = fmaxf(amax, fabsf(v.hi));
    }
    if (valid4) {
#pragma unroll
      for (int cc = 0; cc < 16; ++cc) {
        const int c = 16 * qq + cc;
        if (c < nb) {
          if (rho4 < T)
            Lf[koff + (int64_t)(c0 + c) * m + c0 + nb + rho4] = pv[cc];
          else
            G[qoff + (rho4 - T) * m + c0 + c] = pv[cc];
        }
      }
    }
    amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, 1));
    amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, 2));
    const int e = tc::row_exponent(amax);
    if (qq == 0) ex[rho4] = e;
#pragma unroll
    for (int g = 0; g < 2; ++g) {
      ff xg[8];
#pragma unroll
      for (int cc = 0; cc < 8; ++cc) xg[cc] = pv[8 * g + cc];
      store_slices8(sl, RP, rho4, 2 * qq + g, xg, e);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (w == 0) tc::tmem_dealloc(tmem, kLcTmemCols);
}

// ---------------------------------------------------------------------------------------------
// Trailing update step: grid = (nleaf, row tiles, column tiles), block = kLcTcThreads.
// Shared memory: kSlices A slices (kATileBytes each), then kSlices B slices (kBTileBytes each).
// A thread updates 16 entries of C (tile row 32 (w % 4) + lane, columns 16 (w / 4) .. + 15),
// loading the first eight while the products run and the next eight one chunk ahead.
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kLcTcThreads, 1) k_lc_update(ff* __restrict__ Lf, ff* __restrict__ G, int r,
                                                               DTree t, int c0, const uint16_t* __restrict__ slices,
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
  }
  const int q = w & 3, h = w >> 2;
  const int64_t rho = (int64_t)kLcTileM * rt + 32 * q + lane;
  const bool rvalid = rho < R;
  const int erow = rvalid ? ex[rho] : 0;
  auto c_index = [&](int j) -> int64_t {  // -1: not updated by this thread
    if (!rvalid || j >= T || (rho < T && rho < j)) return -1;
    return rho < T ? koff + (int64_t)(c0 + nb + j) * m + c0 + nb + rho : qoff + (rho - T) * m + c0 + nb + j;
  };
  auto c_load = [&](int64_t o) -> ff {
    if (o < 0) return ff(0.0);
    return rho < T ? Lf[o] : G[o];
  };
  ff cbuf[8];
#pragma unroll
  for (int jj = 0; jj < 8; ++jj) cbuf[jj] = c_load(c_index(kLcTileN * ct + 16 * h + jj));
  if (tid == 0) {
    if (tc::mbar_wait(&bar[0], 0, kTcWaitLimit)) {
      tc::tc_fence_after();
      lc_issue_products(tmem, smA, smB);
    } else {
      serr = 1;
    }
    tc::mma_commit(&bar[1]);
  }
  __syncwarp();
  if (!tc::mbar_wait(&bar[1], 0, kTcWaitLimit)) atomicExch(&serr, 1);
  tc::tc_fence_after();
  __syncthreads();  // serr is the same in every thread from here on
  if (serr) {
    if (tid == 0) {  // copies and products still in flight finish before the exit
      tc::mbar_wait(&bar[0], 0, kTcWaitLimit);
      tc::mbar_wait(&bar[1], 0, kTcWaitLimit);
      info[leaf] = -1;
    }
  } else {
    const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
#pragma unroll 1
    for (int cc = 0; cc < 2; ++cc) {
      const int j0 = 16 * h + 8 * cc;
      ff nbuf[8];
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) nbuf[jj] = cc == 0 ? c_load(c_index(kLcTileN * ct + j0 + 8 + jj)) : ff(0.0);
      ff v[8];
      lc_tile_values(tl, j0, erow, cexp + j0, v);
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        const int64_t o = c_index(kLcTileN * ct + j0 + jj);
        if (o < 0) continue;
        const ff out = cbuf[jj] - v[jj];
        if (rho < T)
          Lf[o] = out;
        else
          G[o] = out;
      }
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) cbuf[jj] = nbuf[jj];
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
__global__ void __launch_bounds__(kLcProbeThreads, 1) k_tc_probe(const double* __restrict__ A,
                                                                 const double* __restrict__ B, int mode,
                                                                 double* __restrict__ C, int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ int rexp[kLcTileM + kLcTileN];
  __shared__ int serr;
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  uint16_t* sA = reinterpret_cast<uint16_t*>(smraw);
  uint16_t* sB = sA + kSlices * kATileBytes / 2;
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_fence_init();
    serr = 0;
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
  if (!tc::mbar_wait(&bar, 0, kTcWaitLimit)) atomicExch(&serr, 1);
  tc::tc_fence_after();
  __syncthreads();  // serr is the same in every thread from here on
  if (serr) {
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

// ---------------------------------------------------------------------------------------------
// Leaf triangular solves with the factor of the tensor-core stage: L x = b (op 0) or L' x = b
// (op 1) by 64-row blocks, x_q = X_q (b_q - L_q,<q x_<q) with X_q the inverse of diagonal block q
// kept by k_lc_diag (strictly lower part in the block's upper triangle, diagonal 1 / D_ii), so
// that both steps are block products spread over all threads: no sequential chain over rows
// (the substitution of k_leaf_tri runs one warp per column through each block).  After x_q the
// remaining rows are updated at once (right-looking).  Same arithmetic as the TC stage's own
// block column products, which use the same inverses.  The block of NC = 4 right-hand sides
// lives in shared memory (narrow chunks keep several CTAs per leaf and SM in flight); grid
// (nleaf, ceil(k / NC)), block 256.
// ---------------------------------------------------------------------------------------------
template <int NC>
__global__ void __launch_bounds__(256) k_leaf_tri_blk(const ff* __restrict__ Lf, DTree t, int op,
                                                      ff* __restrict__ X, int64_t ldx, int k) {
  extern __shared__ __align__(16) unsigned char lc_smem_s[];
  constexpr int LD = kLcNB + 1;
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf), koff = d_leaf_koff(t, leaf);
  const int c0 = blockIdx.y * NC, nc = min(NC, k - c0);
  const int tid = threadIdx.x;
  ff* xs = reinterpret_cast<ff*>(lc_smem_s);  // NC x m, column c at xs[c * m]
  ff* Xq = xs + NC * m;                       // 64 x 65, X_q[i][c] at Xq[i * LD + c]
  for (int e = tid; e < NC * m; e += blockDim.x) {
    const int c = e / m, i = e - c * m;
    xs[e] = c < nc ? X[(int64_t)(c0 + c) * ldx + s + i] : ff(0.0);
  }
  const int nbk = (m + kLcNB - 1) / kLcNB;
  for (int step = 0; step < nbk; ++step) {
    const int q = op == 0 ? step : nbk - 1 - step;
    const int b0 = kLcNB * q, nb = min(kLcNB, m - b0);
    __syncthreads();
    for (int e = tid; e < kLcNB * kLcNB; e += blockDim.x) {
      const int i = e / kLcNB, c = e - i * kLcNB;
      ff v(0.0);
      if (i < nb && c < nb) {
        if (c < i) v = Lf[koff + (int64_t)(b0 + i) * m + b0 + c];
        else if (c == i) v = ff(1.0) / Lf[koff + (int64_t)(b0 + i) * m + b0 + i];
      }
      Xq[i * LD + c] = v;
    }
    __syncthreads();
    // x_q = X_q y_q (op 0) or X_q' y_q (op 1): thread (row i, columns g, g + 4, ...)
    const int i = tid & (kLcNB - 1), g = tid >> 6;
    ff res[NC / 4];
#pragma unroll
    for (int u = 0; u < NC / 4; ++u) {
      const int col = g + 4 * u;
      acc_t<ff> a{};
      if (col < nc && i < nb) {
        const ff* y = xs + col * m + b0;
        if (op == 0)
          for (int c = 0; c < nb; ++c) a += Xq[i * LD + c] * y[c];
        else
          for (int c = 0; c < nb; ++c) a += Xq[c * LD + i] * y[c];
      }
      res[u] = accv(a);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < NC / 4; ++u) {
      const int col = g + 4 * u;
      if (col < nc && i < nb) xs[col * m + b0 + i] = res[u];
    }
    __syncthreads();
    // remaining rows: op 0 rows below the block, op 1 rows above it
    const int r0 = op == 0 ? b0 + nb : 0, r1 = op == 0 ? m : b0;
    for (int row = r0 + tid; row < r1; row += blockDim.x) {
      acc_t<ff> a[NC] = {};
      int l = 0;
      for (; l + 3 < nb; l += 4) {  // four entries of L loaded ahead of their multiply-adds
        ff lv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          lv[u] = op == 0 ? Lf[koff + (int64_t)(b0 + l + u) * m + row] : Lf[koff + (int64_t)row * m + b0 + l + u];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int c = 0; c < NC; ++c)
            if (c < nc) a[c] += lv[u] * xs[c * m + b0 + l + u];
      }
      for (; l < nb; ++l) {
        const ff lv = op == 0 ? Lf[koff + (int64_t)(b0 + l) * m + row] : Lf[koff + (int64_t)row * m + b0 + l];
#pragma unroll
        for (int c = 0; c < NC; ++c)
          if (c < nc) a[c] += lv * xs[c * m + b0 + l];
      }
#pragma unroll
      for (int c = 0; c < NC; ++c)
        if (c < nc) xs[c * m + row] -= accv(a[c]);
    }
  }
  __syncthreads();
  for (int e = tid; e < nc * m; e += blockDim.x) {
    const int c = e / m, i = e - c * m;
    X[(int64_t)(c0 + c) * ldx + s + i] = xs[e];
  }
}

template <int NC>
static bool tri_blk_launch(const ff* Lf, const Tree& t, int op, ff* X, int64_t ldx, int k, cudaStream_t st) {
  const size_t sm = ((size_t)NC * t.max_leaf + (size_t)kLcNB * (kLcNB + 1)) * sizeof(ff);
  if (sm > 200 * 1024) return false;
  smem_limit((const void*)k_leaf_tri_blk<NC>, sm);
  k_leaf_tri_blk<NC><<<dim3((unsigned)t.nleaf, (unsigned)((k + NC - 1) / NC)), 256, sm, st>>>(Lf, dtree(t), op, X,
                                                                                              ldx, k);
  return true;
}

bool launch_leaf_tri_blk(const ff* Lf, const Tree& t, int op, ff* X, int64_t ldx, int k, cudaStream_t st) {
  if (k <= 0) return true;
  if (t.max_leaf > kLcMaxLeaf || (op != 0 && op != 1)) return false;
  return tri_blk_launch<4>(Lf, t, op, X, ldx, k, st);
}

bool leaf_chol_tc_supported(const Tree& t, int r) {
  return t.max_leaf >= 1 && t.max_leaf <= kLcMaxLeaf && r >= 1 && r <= kLcMaxRank;
}

// Scratch per leaf: the slices of the rows below the block (kSlices x RP x 64 bf16) and of X
// (kSlices x 64 x 64 bf16), then the row exponents of both.
int64_t leaf_chol_tc_scratch_bytes(const Tree& t, int r) {
  const int64_t rp = lc_rp_max(t, r);
  return t.nleaf * ((rp * kLcNB + (int64_t)kLcNB * kLcNB) * kSlices * (int64_t)sizeof(uint16_t) +
                    (rp + kLcNB) * (int64_t)sizeof(int));
}

int leaf_chol_tc_steps(const Tree& t) { return (int)((t.max_leaf + kLcNB - 1) / kLcNB); }

bool leaf_chol_tc_has_update(const Tree& t, int p) { return t.max_leaf - (int64_t)kLcNB * (p + 1) > 0; }

struct LcArgs {
  uint16_t* slices;
  uint16_t* xsl;
  int* rexp;
  int* xexp;
  int64_t slice_stride, exp_stride;
};

static LcArgs lc_args(const Tree& t, int r, void* scratch) {
  const int64_t rp = lc_rp_max(t, r);
  LcArgs a;
  a.slice_stride = rp * kLcNB * kSlices;
  a.exp_stride = rp;
  a.slices = reinterpret_cast<uint16_t*>(scratch);
  a.xsl = a.slices + t.nleaf * a.slice_stride;
  a.rexp = reinterpret_cast<int*>(a.xsl + t.nleaf * (int64_t)kSlices * kLcNB * kLcNB);
  a.xexp = a.rexp + t.nleaf * rp;
  return a;
}

void launch_leaf_chol_tc_diag(ff* Lf, int r, const Tree& t, int p, void* scratch, int* info, cudaStream_t st) {
  const LcArgs a = lc_args(t, r, scratch);
  const size_t smd = (size_t)2 * kLcNB * (kLcNB + 1) * sizeof(ff);
  smem_limit((const void*)k_lc_diag, smd);
  k_lc_diag<<<(unsigned)t.nleaf, kLcDiagThreads, smd, st>>>(Lf, dtree(t), kLcNB * p, a.xsl, a.xexp, info);
}

void launch_leaf_chol_tc_trsm(ff* Lf, ff* G, int r, const Tree& t, int p, void* scratch, int* info,
                              cudaStream_t st) {
  const LcArgs a = lc_args(t, r, scratch);
  const int c0 = kLcNB * p;
  const size_t sm = (size_t)kSlices * (kATileBytes + kBTileBytes);
  smem_limit((const void*)k_lc_trsm, sm);
  const int64_t rmax = t.max_leaf - c0 - 1 + r;  // rows below the block of the largest leaf, nb >= 1
  dim3 grid((unsigned)t.nleaf, (unsigned)((rmax + kLcTileM - 1) / kLcTileM));
  k_lc_trsm<<<grid, kLcTcThreads, sm, st>>>(Lf, G, r, dtree(t), c0, a.xsl, a.xexp, a.slices, a.rexp, a.slice_stride,
                                            a.exp_stride, info);
}

void launch_leaf_chol_tc_update(ff* Lf, ff* G, int r, const Tree& t, int p, void* scratch, int* info,
                                cudaStream_t st) {
  const LcArgs a = lc_args(t, r, scratch);
  const size_t sm = (size_t)kSlices * (kATileBytes + kBTileBytes);
  const int c0 = kLcNB * p;
  const int64_t tmax = t.max_leaf - c0 - kLcNB;
  if (tmax <= 0) return;
  dim3 grid((unsigned)t.nleaf, (unsigned)((tmax + r + kLcTileM - 1) / kLcTileM),
            (unsigned)((tmax + kLcTileN - 1) / kLcTileN));
  smem_limit((const void*)k_lc_update, sm);
  k_lc_update<<<grid, kLcTcThreads, sm, st>>>(Lf, G, r, dtree(t), c0, a.slices, a.rexp, a.slice_stride,
                                              a.exp_stride, info);
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
    k_tc_probe<<<1, kLcProbeThreads, smu>>>(dA, dB, mode, dC, dst);
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
