// Leaf-level kernels: triangular solves/products with the leaf Cholesky factors and the
// projections Q_leaf' y / expansions Q_leaf g through the leaf Householder reflectors.
//
// These replace the blockwise loops ldiv!/mul!(BDiagonal(leafW), .) of the reference
// (src/HODLR/src/BlockDiagonal.jl:51-70, used by src/HODLR/src/utils.jl:54-65 and
// src/HODLR/src/baseoverloads.jl:95-150).  One CTA handles one leaf and a chunk of right-hand
// sides staged in shared memory; the triangular solves are blocked by 32 rows so that the
// dependency chain is a 32-step shuffle solve per block and the bulk of the work is an
// independent multiply-add update (FP64 throughput bound).
#include "km_kernels.h"

namespace km {

// ---------------------------------------------------------------------------------------------
// Blocked leaf triangular kernels, L lower triangular (column-major m x m):
//   op 0: X = L^{-1} B   op 1: X = L^{-T} B   op 2: X = L B   op 3: X = L^T B
// grid = (nleaf, ceil(ncols / NC)), block = 256.
// ---------------------------------------------------------------------------------------------
template <int NC>
__device__ void leaf_tri_body(const double* __restrict__ L, int m, int op, const double* Bp, int64_t ldb,
                              double* Xp, int64_t ldx, int nc, double* sm) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  double* xs = sm;                   // NC x m  (column c at xs[c*m])
  double* ys = xs + NC * m;          // NC x m  (products only)
  double* D = ys + ((op >= 2) ? NC * m : 0);  // 32 x 33
  for (int e = tid; e < NC * m; e += blockDim.x) {
    const int c = e / m, i = e % m;
    xs[e] = (c < nc) ? Bp[(int64_t)c * ldb + i] : 0.0;
  }
  __syncthreads();
  if (op == 0 || op == 1) {
    const int nblk = (m + 31) / 32;
    for (int q = 0; q < nblk; ++q) {
      const int i0 = (op == 0) ? q * 32 : (nblk - 1 - q) * 32;
      const int ib = min(32, m - i0);
      for (int e = tid; e < 32 * 32; e += blockDim.x) {
        const int i = e & 31, l = e >> 5;
        if (i < ib && l <= i) D[i * 33 + l] = L[(int64_t)(i0 + l) * m + i0 + i];
      }
      __syncthreads();
      // diagonal block, one warp per column, lanes = rows of the block
      for (int c = w; c < nc; c += 8) {
        double x = (lane < ib) ? xs[c * m + i0 + lane] : 0.0;
        if (op == 0) {
          for (int l = 0; l < ib; ++l) {
            if (lane == l) x = x / D[l * 33 + l];
            const double xl = __shfl_sync(0xffffffffu, x, l);
            if (lane > l && lane < ib) x -= D[lane * 33 + l] * xl;
          }
        } else {
          for (int l = ib - 1; l >= 0; --l) {
            if (lane == l) x = x / D[l * 33 + l];
            const double xl = __shfl_sync(0xffffffffu, x, l);
            if (lane < l) x -= D[l * 33 + lane] * xl;
          }
        }
        if (lane < ib) xs[c * m + i0 + lane] = x;
      }
      __syncthreads();
      // update of the remaining rows with the solved block (thread per row, NC accumulators)
      if (op == 0) {
        for (int i = i0 + ib + tid; i < m; i += blockDim.x) {
          double acc[NC];
#pragma unroll
          for (int c = 0; c < NC; ++c) acc[c] = 0.0;
          for (int l = 0; l < ib; ++l) {
            const double a = L[(int64_t)(i0 + l) * m + i];
#pragma unroll
            for (int c = 0; c < NC; ++c) acc[c] += a * xs[c * m + i0 + l];
          }
#pragma unroll
          for (int c = 0; c < NC; ++c) xs[c * m + i] -= acc[c];
        }
      } else {
        for (int i = tid; i < i0; i += blockDim.x) {
          double acc[NC];
#pragma unroll
          for (int c = 0; c < NC; ++c) acc[c] = 0.0;
          const double* col = L + (int64_t)i * m + i0;  // L[i0 + l, i]
          for (int l = 0; l < ib; ++l) {
            const double a = col[l];
#pragma unroll
            for (int c = 0; c < NC; ++c) acc[c] += a * xs[c * m + i0 + l];
          }
#pragma unroll
          for (int c = 0; c < NC; ++c) xs[c * m + i] -= acc[c];
        }
      }
      __syncthreads();
    }
    for (int e = tid; e < nc * m; e += blockDim.x) {
      const int c = e / m, i = e % m;
      Xp[(int64_t)c * ldx + i] = xs[e];
    }
  } else {
    for (int i = tid; i < m; i += blockDim.x) {
      double acc[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[c] = 0.0;
      if (op == 2) {  // row i of L: L[i, l], l <= i
        for (int l = 0; l <= i; ++l) {
          const double a = L[(int64_t)l * m + i];
#pragma unroll
          for (int c = 0; c < NC; ++c) acc[c] += a * xs[c * m + l];
        }
      } else {        // row i of L^T = column i of L, rows l >= i
        const double* col = L + (int64_t)i * m;
        for (int l = i; l < m; ++l) {
          const double a = col[l];
#pragma unroll
          for (int c = 0; c < NC; ++c) acc[c] += a * xs[c * m + l];
        }
      }
#pragma unroll
      for (int c = 0; c < NC; ++c) ys[c * m + i] = acc[c];
    }
    __syncthreads();
    for (int e = tid; e < nc * m; e += blockDim.x) {
      const int c = e / m, i = e % m;
      Xp[(int64_t)c * ldx + i] = ys[e];
    }
  }
}

template <int NC>
__global__ void __launch_bounds__(256) k_leaf_tri(const double* __restrict__ Lf, DTree t, int op,
                                                  LeafOperand B, LeafOperand X, int ncols) {
  extern __shared__ double sm[];
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int c0 = blockIdx.y * NC;
  const int nc = min(NC, ncols - c0);
  const int64_t ldb = B.ld_is_m ? m : B.ld, ldx = X.ld_is_m ? m : X.ld;
  leaf_tri_body<NC>(Lf + d_leaf_koff(t, leaf), m, op, B.ptr + s * B.bmul + (int64_t)c0 * ldb, ldb,
                    X.ptr + s * X.bmul + (int64_t)c0 * ldx, ldx, nc, sm);
}

// Same operation on arbitrary column blocks: descriptor d covers leaf d.leaf's rows of a block.
template <int NC>
__global__ void __launch_bounds__(256) k_leaf_tri_desc(const double* __restrict__ Lf, DTree t, int op,
                                                       const LeafDesc* __restrict__ descs) {
  extern __shared__ double sm[];
  const LeafDesc d = descs[blockIdx.x];
  const int c0 = blockIdx.y * NC;
  if (c0 >= d.ncols) return;
  const int nc = min(NC, d.ncols - c0);
  const int m = d_leaf_size(t, d.leaf);
  double* p = d.ptr + (int64_t)c0 * d.ld;
  leaf_tri_body<NC>(Lf + d_leaf_koff(t, d.leaf), m, op, p, d.ld, p, d.ld, nc, sm);
}


// ---------------------------------------------------------------------------------------------
// Q_leaf' y  (proj) and y += sign * Q_leaf g (expand) through the leaf reflectors.
// grid = (nleaf, ceil(k / 16)), block 256: warp w owns columns w and w+8 of the chunk.
// SMEMV: the leaf's reflectors (m x r) are staged in shared memory.
// ---------------------------------------------------------------------------------------------
template <bool SMEMV, bool EXPAND>
__global__ void __launch_bounds__(256) k_leaf_refl(const double* __restrict__ Qref, const double* __restrict__ tau,
                                                   int r, DTree t, const double* __restrict__ VG,
                                                   double* __restrict__ Y, int64_t ldy,
                                                   double* __restrict__ VP, int k, double sign) {
  extern __shared__ double sm[];
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int c0 = blockIdx.y * 16;
  const int nc = min(16, k - c0);
  double* ys = sm;                 // 16 x m
  double* ts = ys + 16 * m;        // r
  double* Vs = ts + r;             // m x r when SMEMV
  const double* Qg = Qref + s * r;
  const double* V = SMEMV ? Vs : Qg;
  if (SMEMV)
    for (int64_t e = tid; e < (int64_t)m * r; e += blockDim.x) Vs[e] = Qg[e];
  for (int e = tid; e < r; e += blockDim.x) ts[e] = tau[leaf * r + e];
  for (int e = tid; e < 16 * m; e += blockDim.x) {
    const int c = e / m, i = e % m;
    double v = 0.0;
    if (c < nc) {
      if (EXPAND) v = (i < r) ? VG[(leaf * k + c0 + c) * r + i] : 0.0;
      else v = Y[(int64_t)(c0 + c) * ldy + s + i];
    }
    ys[e] = v;
  }
  __syncthreads();
  const int ca = w, cb = w + 8;
  const bool hb = cb < nc;
  if (ca < nc) {
    double* ya = ys + ca * m;
    double* yb = ys + cb * m;
    for (int q = 0; q < r; ++q) {
      const int j = EXPAND ? r - 1 - q : q;
      const double tj = ts[j];
      if (tj == 0.0) continue;
      const double* v = V + (int64_t)j * m;
      double aa = 0.0, ab = 0.0;
      for (int i = j + 1 + lane; i < m; i += 32) {
        const double vi = v[i];
        aa += vi * ya[i];
        if (hb) ab += vi * yb[i];
      }
      aa = warp_sum(aa);
      ab = warp_sum(ab);
      aa = (aa + ya[j]) * tj;
      ab = hb ? (ab + yb[j]) * tj : 0.0;
      __syncwarp();
      if (lane == 0) {
        ya[j] -= aa;
        if (hb) yb[j] -= ab;
      }
      for (int i = j + 1 + lane; i < m; i += 32) {
        const double vi = v[i];
        ya[i] -= aa * vi;
        if (hb) yb[i] -= ab * vi;
      }
      __syncwarp();
    }
  }
  __syncthreads();
  if (EXPAND) {
    for (int e = tid; e < nc * m; e += blockDim.x) {
      const int c = e / m, i = e % m;
      Y[(int64_t)(c0 + c) * ldy + s + i] += sign * ys[e];
    }
  } else {
    for (int e = tid; e < nc * r; e += blockDim.x) {
      const int c = e / r, i = e % r;
      VP[(leaf * k + c0 + c) * r + i] = ys[c * m + i];
    }
  }
}

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
template <int NC>
static bool tri_launch(const double* Lf, const Tree& t, int op, LeafOperand B, LeafOperand X, int ncols,
                       cudaStream_t st) {
  const size_t sm = ((size_t)(op >= 2 ? 2 : 1) * NC * t.max_leaf + 32 * 33) * sizeof(double);
  if (sm > 200 * 1024) return false;
  cudaFuncSetAttribute(k_leaf_tri<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid((unsigned)t.nleaf, (unsigned)((ncols + NC - 1) / NC));
  k_leaf_tri<NC><<<grid, 256, sm, st>>>(Lf, dtree(t), op, B, X, ncols);
  return true;
}

bool launch_leaf_tri(const double* Lf, const Tree& t, int op, double* Bptr, int64_t bmul,
                     int64_t bld, int bld_is_m, double* Xptr, int64_t xmul, int64_t xld,
                     int xld_is_m, int ncols, cudaStream_t st) {
  LeafOperand B{Bptr, bmul, bld, bld_is_m}, X{Xptr, xmul, xld, xld_is_m};
  if (ncols > 8 && tri_launch<16>(Lf, t, op, B, X, ncols, st)) return true;
  if (tri_launch<8>(Lf, t, op, B, X, ncols, st)) return true;
  if (tri_launch<4>(Lf, t, op, B, X, ncols, st)) return true;
  return tri_launch<1>(Lf, t, op, B, X, ncols, st);
}

template <int NC>
static bool tri_desc_launch(const double* Lf, const Tree& t, int op, const LeafDesc* descs, int n, int maxcols,
                            cudaStream_t st) {
  const size_t sm = ((size_t)(op >= 2 ? 2 : 1) * NC * t.max_leaf + 32 * 33) * sizeof(double);
  if (sm > 200 * 1024) return false;
  cudaFuncSetAttribute(k_leaf_tri_desc<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid((unsigned)n, (unsigned)((maxcols + NC - 1) / NC));
  k_leaf_tri_desc<NC><<<grid, 256, sm, st>>>(Lf, dtree(t), op, descs);
  return true;
}

bool launch_leaf_tri_desc(const double* Lf, const Tree& t, int op, const LeafDesc* descs, int n, int maxcols,
                          cudaStream_t st) {
  if (n <= 0) return true;
  if (tri_desc_launch<16>(Lf, t, op, descs, n, maxcols, st)) return true;
  if (tri_desc_launch<8>(Lf, t, op, descs, n, maxcols, st)) return true;
  if (tri_desc_launch<4>(Lf, t, op, descs, n, maxcols, st)) return true;
  return tri_desc_launch<1>(Lf, t, op, descs, n, maxcols, st);
}

template <bool EXPAND>
static void refl_launch(const double* Qref, const double* tau, int r, const Tree& t, const double* VG,
                        double* Y, int64_t ldy, double* VP, int k, double sign, cudaStream_t st) {
  dim3 grid((unsigned)t.nleaf, (unsigned)((k + 15) / 16));
  const size_t base = ((size_t)16 * t.max_leaf + r) * sizeof(double);
  const size_t full = base + (size_t)t.max_leaf * r * sizeof(double);
  if (full <= 200 * 1024) {
    cudaFuncSetAttribute(k_leaf_refl<true, EXPAND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)full);
    k_leaf_refl<true, EXPAND><<<grid, 256, full, st>>>(Qref, tau, r, dtree(t), VG, Y, ldy, VP, k, sign);
  } else {
    cudaFuncSetAttribute(k_leaf_refl<false, EXPAND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)base);
    k_leaf_refl<false, EXPAND><<<grid, 256, base, st>>>(Qref, tau, r, dtree(t), VG, Y, ldy, VP, k, sign);
  }
}

void launch_leaf_proj(const double* Qref, const double* tau, int r, const Tree& t, const double* Y,
                      int64_t ldy, double* VP, int k, cudaStream_t st) {
  refl_launch<false>(Qref, tau, r, t, nullptr, const_cast<double*>(Y), ldy, VP, k, 0.0, st);
}

void launch_leaf_expand(const double* Qref, const double* tau, int r, const Tree& t, const double* VG,
                        double* Y, int64_t ldy, int k, double sign, cudaStream_t st) {
  refl_launch<true>(Qref, tau, r, t, VG, Y, ldy, nullptr, k, sign, st);
}

}  // namespace km
