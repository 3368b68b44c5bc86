// FP64 products of the general (ACA) factorisation: C = alpha op(A) B + beta C, column-major,
// op(A) = A or A'.  They replace the dense BLAS calls of the reference's per-block updates
// (the `mul!` products of symfact.jl:28-38 and of the panel QR in lrsymfact, utils.jl:29-35) for
// the blocks of 16384 rows or more: projections Q' x and V' C (op = T, a long reduction over the
// rows), expansions Q g and C - V W (op = N, many rows, a short reduction) and the small block
// reflector products op(T) W.
//
// GB300 issues 2 FP64 FMAs per clock per SM, so these products are bound by the FP64 pipe, not by
// memory or shared-memory traffic: the kernels only have to avoid wasted multiply-adds and keep
// enough warps in flight.  A CTA computes a tile of 1024 outputs whose shape follows the operands
// (8 x 128 when op(A) has at most 8 rows, 128 x 8 when B has at most 8 columns, 32 x 32
// otherwise), staging 32-deep slices of op(A) and B in shared memory with coalesced loads; each
// thread owns 4 outputs.  Long reductions (op = T with many rows) are split over grid.z: every
// CTA writes its partial tile and a second kernel adds the partials in a fixed order, so results
// do not depend on scheduling.
#include <algorithm>

#include "km_kernels.h"

namespace km {

constexpr int kGK = 32;  // reduction depth staged per step

template <int TM, int TN, bool TRANS>
__global__ void __launch_bounds__(256) k_dgemm(int64_t M, int64_t N, int64_t K, int64_t kchunk, double alpha,
                                               const double* __restrict__ A, int64_t lda,
                                               const double* __restrict__ B, int64_t ldb, double beta,
                                               double* __restrict__ C, int64_t ldc, double* __restrict__ part) {
  __shared__ double As[kGK][TM + 1];
  __shared__ double Bs[kGK][TN + 1];
  const int64_t m0 = (int64_t)blockIdx.x * TM, n0 = (int64_t)blockIdx.y * TN;
  const int64_t k0 = (int64_t)blockIdx.z * kchunk, k1 = (K < k0 + kchunk) ? K : k0 + kchunk;
  const int tid = threadIdx.x;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  int om[4], on[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int o = tid + 256 * q;
    om[q] = o % TM;
    on[q] = o / TM;
  }
  for (int64_t kb = k0; kb < k1; kb += kGK) {
    const int kd = (int)((k1 - kb < kGK) ? k1 - kb : kGK);
    __syncthreads();
    for (int e = tid; e < kGK * TM; e += 256) {
      int k, m;
      if (TRANS) {  // A is K x M: (k, m) at A[k + m lda], rows k contiguous
        k = e % kGK;
        m = e / kGK;
      } else {      // A is M x K: (m, k) at A[m + k lda], rows m contiguous
        m = e % TM;
        k = e / TM;
      }
      const int64_t gm = m0 + m, gk = kb + k;
      double v = 0.0;
      if (k < kd && gm < M) v = TRANS ? A[gk + gm * lda] : A[gm + gk * lda];
      As[k][m] = v;
    }
    for (int e = tid; e < kGK * TN; e += 256) {
      const int k = e % kGK, n = e / kGK;
      const int64_t gn = n0 + n, gk = kb + k;
      Bs[k][n] = (k < kd && gn < N) ? B[gk + gn * ldb] : 0.0;
    }
    __syncthreads();
    for (int k = 0; k < kd; ++k)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = fma(As[k][om[q]], Bs[k][on[q]], acc[q]);
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int64_t gm = m0 + om[q], gn = n0 + on[q];
    if (gm >= M || gn >= N) continue;
    if (part) {
      part[((int64_t)blockIdx.z * N + gn) * M + gm] = acc[q];
    } else {
      const double c = (beta == 0.0) ? 0.0 : beta * C[gm + gn * ldc];
      C[gm + gn * ldc] = alpha * acc[q] + c;
    }
  }
}

// C = alpha sum_z part[z] + beta C, z in order
__global__ void k_dgemm_reduce(int64_t M, int64_t N, int S, double alpha, const double* __restrict__ part,
                               double beta, double* __restrict__ C, int64_t ldc) {
  const int64_t MN = M * N;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < MN; e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int z = 0; z < S; ++z) s += part[z * MN + e];
    const int64_t m = e % M, n = e / M;
    const double c = (beta == 0.0) ? 0.0 : beta * C[m + n * ldc];
    C[m + n * ldc] = alpha * s + c;
  }
}

// split of the reduction: chunks of at least 2048 rows, about 4 CTAs per SM over all tiles
static int dgemm_splits(int64_t tiles, int64_t K) {
  const int64_t want = std::max<int64_t>(1, (4 * 152) / std::max<int64_t>(tiles, 1));
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (K + 2047) / 2048));
}

static void tile_shape(int64_t M, int64_t N, int* tm, int* tn) {
  if (M <= 8) {
    *tm = 8;
    *tn = 128;
  } else if (N <= 8) {
    *tm = 128;
    *tn = 8;
  } else {
    *tm = 32;
    *tn = 32;
  }
}

int64_t dgemm_scratch(int transA, int64_t M, int64_t N, int64_t K) {
  if (!transA || M <= 0 || N <= 0) return 0;
  int tm, tn;
  tile_shape(M, N, &tm, &tn);
  const int64_t tiles = ((M + tm - 1) / tm) * ((N + tn - 1) / tn);
  const int S = dgemm_splits(tiles, K);
  return S > 1 ? (int64_t)S * M * N : 0;
}

template <int TM, int TN>
static void dgemm_launch(int transA, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                         const double* B, int64_t ldb, double beta, double* C, int64_t ldc, double* scratch,
                         int64_t scratch_len, cudaStream_t st) {
  const int64_t gm = (M + TM - 1) / TM, gn = (N + TN - 1) / TN;
  int S = (transA && scratch) ? dgemm_splits(gm * gn, K) : 1;
  S = (int)std::max<int64_t>(1, std::min<int64_t>(S, scratch_len / (M * N)));
  const int64_t kchunk = (S > 1) ? ((K + S - 1) / S + kGK - 1) / kGK * kGK : std::max<int64_t>(K, 1);
  const int Sz = (int)((K + kchunk - 1) / kchunk);
  double* part = (Sz > 1) ? scratch : nullptr;
  dim3 grid((unsigned)gm, (unsigned)gn, (unsigned)std::max(Sz, 1));
  if (transA)
    k_dgemm<TM, TN, true><<<grid, 256, 0, st>>>(M, N, K, kchunk, alpha, A, lda, B, ldb, beta, C, ldc, part);
  else
    k_dgemm<TM, TN, false><<<grid, 256, 0, st>>>(M, N, K, kchunk, alpha, A, lda, B, ldb, beta, C, ldc, part);
  if (part) {
    const int64_t MN = M * N;
    k_dgemm_reduce<<<(unsigned)std::min<int64_t>((MN + 255) / 256, 4096), 256, 0, st>>>(M, N, Sz, alpha, part,
                                                                                        beta, C, ldc);
  }
}

void launch_dgemm(int transA, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                  const double* B, int64_t ldb, double beta, double* C, int64_t ldc, double* scratch,
                  int64_t scratch_len, cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  int tm, tn;
  tile_shape(M, N, &tm, &tn);
  if (tm == 8)
    dgemm_launch<8, 128>(transA, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, scratch, scratch_len, st);
  else if (tn == 8)
    dgemm_launch<128, 8>(transA, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, scratch, scratch_len, st);
  else
    dgemm_launch<32, 32>(transA, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, scratch, scratch_len, st);
}

}  // namespace km
