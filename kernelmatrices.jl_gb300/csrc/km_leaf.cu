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
template <typename T, int NC>
__device__ void leaf_tri_body(const T* __restrict__ L, int m, int op, const T* Bp, int64_t ldb, T* Xp,
                              int64_t ldx, int nc, T* sm) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  T* xs = sm;                   // NC x m  (column c at xs[c*m])
  T* ys = xs + NC * m;          // NC x m  (products only)
  T* D = ys + ((op >= 2) ? NC * m : 0);  // 32 x 33
  for (int e = tid; e < NC * m; e += blockDim.x) {
    const int c = e / m, i = e % m;
    xs[e] = (c < nc) ? Bp[(int64_t)c * ldb + i] : T(0.0);
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
        T x = (lane < ib) ? xs[c * m + i0 + lane] : T(0.0);
        if (op == 0) {
          for (int l = 0; l < ib; ++l) {
            if (lane == l) x = x / D[l * 33 + l];
            const T xl = shfl_idx(x, l);
            if (lane > l && lane < ib) x -= D[lane * 33 + l] * xl;
          }
        } else {
          for (int l = ib - 1; l >= 0; --l) {
            if (lane == l) x = x / D[l * 33 + l];
            const T xl = shfl_idx(x, l);
            if (lane < l) x -= D[l * 33 + lane] * xl;
          }
        }
        if (lane < ib) xs[c * m + i0 + lane] = x;
      }
      __syncthreads();
      // update of the remaining rows with the solved block (thread per row, NC accumulators)
      if (op == 0) {
        for (int i = i0 + ib + tid; i < m; i += blockDim.x) {
          T acc[NC];
#pragma unroll
          for (int c = 0; c < NC; ++c) acc[c] = T(0.0);
          for (int l = 0; l < ib; ++l) {
            const T a = L[(int64_t)(i0 + l) * m + i];
#pragma unroll
            for (int c = 0; c < NC; ++c) acc[c] += a * xs[c * m + i0 + l];
          }
#pragma unroll
          for (int c = 0; c < NC; ++c) xs[c * m + i] -= acc[c];
        }
      } else {
        for (int i = tid; i < i0; i += blockDim.x) {
          T acc[NC];
#pragma unroll
          for (int c = 0; c < NC; ++c) acc[c] = T(0.0);
          const T* col = L + (int64_t)i * m + i0;  // L[i0 + l, i]
          for (int l = 0; l < ib; ++l) {
            const T a = col[l];
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
      T acc[NC];
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[c] = T(0.0);
      if (op == 2) {  // row i of L: L[i, l], l <= i
        for (int l = 0; l <= i; ++l) {
          const T a = L[(int64_t)l * m + i];
#pragma unroll
          for (int c = 0; c < NC; ++c) acc[c] += a * xs[c * m + l];
        }
      } else {        // row i of L^T = column i of L, rows l >= i
        const T* col = L + (int64_t)i * m;
        for (int l = i; l < m; ++l) {
          const T a = col[l];
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

template <typename T, int NC>
__global__ void __launch_bounds__(256) k_leaf_tri(const T* __restrict__ Lf, DTree t, int op,
                                                  LeafOperand B, LeafOperand X, int ncols) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int c0 = blockIdx.y * NC;
  const int nc = min(NC, ncols - c0);
  const int64_t ldb = B.ld_is_m ? m : B.ld, ldx = X.ld_is_m ? m : X.ld;
  leaf_tri_body<T, NC>(Lf + d_leaf_koff(t, leaf), m, op,
                       reinterpret_cast<const T*>(B.ptr) + s * B.bmul + (int64_t)c0 * ldb, ldb,
                       reinterpret_cast<T*>(X.ptr) + s * X.bmul + (int64_t)c0 * ldx, ldx, nc, sm);
}

// Same operation on arbitrary column blocks: descriptor d covers leaf d.leaf's rows of a block.
template <int NC>
__global__ void __launch_bounds__(256) k_leaf_tri_desc(const double* __restrict__ Lf, DTree t, int op,
                                                       const LeafDesc* __restrict__ descs) {
  extern __shared__ __align__(16) unsigned char smraw[];
  double* sm = reinterpret_cast<double*>(smraw);
  const LeafDesc d = descs[blockIdx.x];
  const int c0 = blockIdx.y * NC;
  if (c0 >= d.ncols) return;
  const int nc = min(NC, d.ncols - c0);
  const int m = d_leaf_size(t, d.leaf);
  double* p = d.ptr + (int64_t)c0 * d.ld;
  leaf_tri_body<double, NC>(Lf + d_leaf_koff(t, d.leaf), m, op, p, d.ld, p, d.ld, nc, sm);
}


// ---------------------------------------------------------------------------------------------
// Q_leaf' y (proj) and y += sign * Q_leaf g (expand) with the explicit leaf bases Q (m x r,
// column-major at start*r).  grid = (nleaf, ceil(k / 16)), block 256; the 16-column chunk of y
// (proj) or of g (expand) is staged in shared memory and every output is an independent dot
// product.
// ---------------------------------------------------------------------------------------------
// sum_l a[l*sa] b[l], l < n, with four independent partial sums
template <typename T>
__device__ __forceinline__ T dot4l(const T* __restrict__ a, int64_t sa, const T* __restrict__ b, int n) {
  T s0 = T(0.0), s1 = T(0.0), s2 = T(0.0), s3 = T(0.0);
  int l = 0;
  for (; l + 3 < n; l += 4) {
    s0 += a[l * sa] * b[l];
    s1 += a[(l + 1) * sa] * b[l + 1];
    s2 += a[(l + 2) * sa] * b[l + 2];
    s3 += a[(l + 3) * sa] * b[l + 3];
  }
  for (; l < n; ++l) s0 += a[l * sa] * b[l];
  return (s0 + s1) + (s2 + s3);
}

template <typename T>
__global__ void __launch_bounds__(256) k_leaf_qproj(const T* __restrict__ Q, int r, DTree t, const T* __restrict__ Y,
                                                    int64_t ldy, T* __restrict__ VP, int k) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* ys = reinterpret_cast<T*>(smraw);  // 16 x m
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int c0 = blockIdx.y * 16;
  const int nc = min(16, k - c0);
  for (int e = threadIdx.x; e < nc * m; e += blockDim.x) {
    const int c = e / m, i = e % m;
    ys[c * m + i] = Y[(int64_t)(c0 + c) * ldy + s + i];
  }
  __syncthreads();
  const T* Ql = Q + s * r;
  for (int e = threadIdx.x; e < nc * r; e += blockDim.x) {
    const int q = e % r, c = e / r;
    VP[(leaf * k + c0 + c) * r + q] = dot4l(Ql + (int64_t)q * m, 1, ys + c * m, m);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_leaf_qexpand(const T* __restrict__ Q, int r, DTree t, const T* __restrict__ VG,
                                                      T* __restrict__ Y, int64_t ldy, int k, double sign) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* gs = reinterpret_cast<T*>(smraw);  // 16 x r
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int c0 = blockIdx.y * 16;
  const int nc = min(16, k - c0);
  for (int e = threadIdx.x; e < nc * r; e += blockDim.x) gs[e] = VG[(leaf * k + c0) * r + e];
  __syncthreads();
  const T* Ql = Q + s * r;
  for (int e = threadIdx.x; e < nc * m; e += blockDim.x) {
    const int i = e % m, c = e / m;
    const T acc = dot4l(Ql + i, m, gs + c * r, r);
    T* y = Y + (int64_t)(c0 + c) * ldy + s + i;
    *y = (sign > 0.0) ? *y + acc : *y - acc;
  }
}

// ---------------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------------
template <typename T, int NC>
static bool tri_launch(const T* Lf, const Tree& t, int op, LeafOperand B, LeafOperand X, int ncols,
                       cudaStream_t st) {
  const size_t sm = ((size_t)(op >= 2 ? 2 : 1) * NC * t.max_leaf + 32 * 33) * sizeof(T);
  if (sm > 200 * 1024) return false;
  smem_limit((const void*)k_leaf_tri<T, NC>, sm);
  dim3 grid((unsigned)t.nleaf, (unsigned)((ncols + NC - 1) / NC));
  k_leaf_tri<T, NC><<<grid, 256, sm, st>>>(Lf, dtree(t), op, B, X, ncols);
  return true;
}

template <typename T>
bool launch_leaf_tri(const T* Lf, const Tree& t, int op, T* Bptr, int64_t bmul, int64_t bld, int bld_is_m, T* Xptr,
                     int64_t xmul, int64_t xld, int xld_is_m, int ncols, cudaStream_t st) {
  LeafOperand B{reinterpret_cast<double*>(Bptr), bmul, bld, bld_is_m};
  LeafOperand X{reinterpret_cast<double*>(Xptr), xmul, xld, xld_is_m};
  if (ncols > 8 && tri_launch<T, 16>(Lf, t, op, B, X, ncols, st)) return true;
  if (tri_launch<T, 8>(Lf, t, op, B, X, ncols, st)) return true;
  if (tri_launch<T, 4>(Lf, t, op, B, X, ncols, st)) return true;
  return tri_launch<T, 1>(Lf, t, op, B, X, ncols, st);
}

template <int NC>
static bool tri_desc_launch(const double* Lf, const Tree& t, int op, const LeafDesc* descs, int n, int maxcols,
                            cudaStream_t st) {
  const size_t sm = ((size_t)(op >= 2 ? 2 : 1) * NC * t.max_leaf + 32 * 33) * sizeof(double);
  if (sm > 200 * 1024) return false;
  smem_limit((const void*)k_leaf_tri_desc<NC>, sm);
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

template <typename T>
void launch_leaf_proj(const T* Q, const T*, int r, const Tree& t, const T* Y, int64_t ldy, T* VP, int k,
                      cudaStream_t st) {
  dim3 grid((unsigned)t.nleaf, (unsigned)((k + 15) / 16));
  const size_t sm = (size_t)16 * t.max_leaf * sizeof(T);
  smem_limit((const void*)k_leaf_qproj<T>, sm);
  k_leaf_qproj<T><<<grid, 256, sm, st>>>(Q, r, dtree(t), Y, ldy, VP, k);
}

template <typename T>
void launch_leaf_expand(const T* Q, const T*, int r, const Tree& t, const T* VG, T* Y, int64_t ldy, int k,
                        double sign, cudaStream_t st) {
  dim3 grid((unsigned)t.nleaf, (unsigned)((k + 15) / 16));
  const size_t sm = (size_t)16 * r * sizeof(T);
  k_leaf_qexpand<T><<<grid, 256, sm, st>>>(Q, r, dtree(t), VG, Y, ldy, k, sign);
}

template bool launch_leaf_tri<double>(const double*, const Tree&, int, double*, int64_t, int64_t, int, double*,
                                      int64_t, int64_t, int, int, cudaStream_t);
template bool launch_leaf_tri<ff>(const ff*, const Tree&, int, ff*, int64_t, int64_t, int, ff*, int64_t, int64_t,
                                  int, int, cudaStream_t);
template void launch_leaf_proj<double>(const double*, const double*, int, const Tree&, const double*, int64_t,
                                       double*, int, cudaStream_t);
template void launch_leaf_proj<ff>(const ff*, const ff*, int, const Tree&, const ff*, int64_t, ff*, int,
                                   cudaStream_t);
template void launch_leaf_expand<double>(const double*, const double*, int, const Tree&, const double*, double*,
                                         int64_t, int, double, cudaStream_t);
template void launch_leaf_expand<ff>(const ff*, const ff*, int, const Tree&, const ff*, ff*, int64_t, int, double,
                                     cudaStream_t);

}  // namespace km
