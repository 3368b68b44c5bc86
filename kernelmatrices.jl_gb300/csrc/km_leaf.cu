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
        if (i < ib && l <= i) {
          const T v = L[(int64_t)(i0 + l) * m + i0 + i];
          D[i * 33 + l] = (l == i) ? T(1.0) / v : v;  // diagonal kept as its reciprocal
        }
      }
      __syncthreads();
      // diagonal block, one warp per column, lanes = rows of the block
      for (int c = w; c < nc; c += 8) {
        acc_t<T> xa = (lane < ib) ? xs[c * m + i0 + lane] : T(0.0);  // row `lane`, updates pending
        T x = T(0.0);                                                  // row `lane`, solved
        if (op == 0) {
          for (int l = 0; l < ib; ++l) {
            if (lane == l) x = accv(xa) * D[l * 33 + l];
            const T xl = shfl_idx(x, l);
            if (lane > l && lane < ib) xa -= D[lane * 33 + l] * xl;
          }
        } else {
          for (int l = ib - 1; l >= 0; --l) {
            if (lane == l) x = accv(xa) * D[l * 33 + l];
            const T xl = shfl_idx(x, l);
            if (lane < l) xa -= D[l * 33 + lane] * xl;
          }
        }
        if (lane < ib) xs[c * m + i0 + lane] = x;
      }
      __syncthreads();
      // update of the remaining rows with the solved block: items of (row, 4 columns), so that
      // each loaded L entry feeds 4 multiply-adds and all threads stay busy as the remaining
      // rows shrink
      const int R = (op == 0) ? m - (i0 + ib) : i0;
      const int r0 = (op == 0) ? i0 + ib : 0;
      const int ng = (nc + 3) >> 2;
      for (int e = tid; e < R * ng; e += blockDim.x) {
        const int g = e / R, i = r0 + (e - g * R), cb = 4 * g;
        const T* xc = xs + cb * m + i0;
        acc_t<T> acc[4] = {};
        auto ld = [&](int l) {
          return (op == 0) ? L[(int64_t)(i0 + l) * m + i]   // L[i, i0 + l]
                           : L[(int64_t)i * m + i0 + l];    // L[i0 + l, i]
        };
        int l = 0;
        for (; l + 3 < ib; l += 4) {  // four entries loaded ahead of their multiply-adds
          const T a0 = ld(l), a1 = ld(l + 1), a2 = ld(l + 2), a3 = ld(l + 3);
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (cb + j < nc) {
              acc[j] += a0 * xc[j * m + l];
              acc[j] += a1 * xc[j * m + l + 1];
              acc[j] += a2 * xc[j * m + l + 2];
              acc[j] += a3 * xc[j * m + l + 3];
            }
        }
        for (; l < ib; ++l) {
          const T a = ld(l);
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (cb + j < nc) acc[j] += a * xc[j * m + l];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (cb + j < nc) xs[(cb + j) * m + i] -= accv(acc[j]);
      }
      __syncthreads();
    }
    for (int e = tid; e < nc * m; e += blockDim.x) {
      const int c = e / m, i = e % m;
      Xp[(int64_t)c * ldx + i] = xs[e];
    }
  } else {
    for (int i = tid; i < m; i += blockDim.x) {
      acc_t<T> acc[NC] = {};
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
      for (int c = 0; c < NC; ++c) ys[c * m + i] = accv(acc[c]);
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
// column-major at start*r).  grid = (nleaf, ceil(k / 16)), block 256.
// ---------------------------------------------------------------------------------------------
// VP[leaf][c] = Q_leaf' y_c for a chunk of up to 16 columns.  The leaf is processed in chunks of
// 64 rows: Q (64 x r, padded rows) and y (16 x 64) are staged in shared memory, then thread t
// owns basis column q = t % r and the columns of group t / r, with up to 6 accumulators.
constexpr int kProjRows = 64;

template <typename T>
__global__ void __launch_bounds__(256) k_leaf_qproj(const T* __restrict__ Q, int r, DTree t, const T* __restrict__ Y,
                                                    int64_t ldy, T* __restrict__ VP, int k) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ldq = r + 1;
  T* qs = reinterpret_cast<T*>(smraw);   // kProjRows x (r + 1): element (i, q) at i * ldq + q
  T* ys = qs + kProjRows * ldq;           // 16 x kProjRows
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int c0 = blockIdx.y * 16;
  const int nc = min(16, k - c0);
  const int tid = threadIdx.x;
  const int G = blockDim.x / r;                 // column groups (>= 3 for r <= 80)
  const int q = tid % r, g = tid / r;
  const int cper = (nc + G - 1) / G;            // <= 6
  const int cb = g * cper, ce = min(nc, cb + cper);
  const bool active = g < G;
  acc_t<T> acc[6] = {};
  const T* Ql = Q + s * r;
  for (int i0 = 0; i0 < m; i0 += kProjRows) {
    const int rows = min(kProjRows, m - i0);
    __syncthreads();
    for (int e = tid; e < rows * r; e += blockDim.x) {
      const int qq = e / rows, i = e - qq * rows;
      qs[i * ldq + qq] = Ql[(int64_t)qq * m + i0 + i];
    }
    for (int e = tid; e < nc * rows; e += blockDim.x) {
      const int c = e / rows, i = e - c * rows;
      ys[c * kProjRows + i] = Y[(int64_t)(c0 + c) * ldy + s + i0 + i];
    }
    __syncthreads();
    if (active) {
      for (int i = 0; i < rows; ++i) {
        const T a = qs[i * ldq + q];
#pragma unroll
        for (int j = 0; j < 6; ++j)
          if (cb + j < ce) acc[j] += a * ys[(cb + j) * kProjRows + i];
      }
    }
  }
  if (active)
#pragma unroll
    for (int j = 0; j < 6; ++j)
      if (cb + j < ce) VP[(leaf * k + c0 + cb + j) * r + q] = accv(acc[j]);
}

// y_c += sign * Q_leaf g_c for a chunk of up to 16 columns: thread per leaf row, the chunk's
// coefficients g (16 x r) in shared memory, one accumulator per column; Q is read once.
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
  const bool add = sign > 0.0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    acc_t<T> acc[16] = {};
    int q = 0;
    for (; q + 1 < r; q += 2) {  // two basis entries loaded ahead of their multiply-adds
      const T a0 = Ql[(int64_t)q * m + i], a1 = Ql[(int64_t)(q + 1) * m + i];
#pragma unroll
      for (int c = 0; c < 16; ++c)
        if (c < nc) {
          acc[c] += a0 * gs[c * r + q];
          acc[c] += a1 * gs[c * r + q + 1];
        }
    }
    for (; q < r; ++q) {
      const T a = Ql[(int64_t)q * m + i];
#pragma unroll
      for (int c = 0; c < 16; ++c)
        if (c < nc) acc[c] += a * gs[c * r + q];
    }
#pragma unroll
    for (int c = 0; c < 16; ++c)
      if (c < nc) {
        T* y = Y + (int64_t)(c0 + c) * ldy + s + i;
        *y = add ? *y + accv(acc[c]) : *y - accv(acc[c]);
      }
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
  // widest column chunk that still gives about four CTAs per SM (each CTA re-reads its leaf's
  // factor, which the L2 serves)
  auto ctas = [&](int nc) { return t.nleaf * (int64_t)((ncols + nc - 1) / nc); };
  const int64_t want = 4 * 152;
  if (ncols > 8 && ctas(16) >= want && tri_launch<T, 16>(Lf, t, op, B, X, ncols, st)) return true;
  if (ncols > 4 && ctas(8) >= want && tri_launch<T, 8>(Lf, t, op, B, X, ncols, st)) return true;
  if (ncols > 1 && tri_launch<T, 4>(Lf, t, op, B, X, ncols, st)) return true;
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
  const size_t sm = ((size_t)kProjRows * (r + 1) + 16 * kProjRows) * sizeof(T);
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
