// Exact derivative of the Nystrom HODLR and the pieces of the stochastic NLL gradient.
//
// Replaces DerivativeHODLR (src/HODLR/src/constructor.jl:66-95), DBlock_mul / DBlock_mul_t
// (src/HODLR/src/utils.jl:76-90) and mul!(target, DK::DerivativeHODLR, src)
// (src/HODLR/src/baseoverloads.jl:216-234).  For the block with rows c2 and columns c1,
//   D[c2, c1] x_c1 = dPhi_c2 S^{-1} phi_c1 - Phi_c2 S^{-1} Sj S^{-1} phi_c1 + Phi_c2 S^{-1} dphi_c1
// with phi = Phi' x, dphi = dPhi' x, Phi = K(X, P), dPhi = dK(X, P), S = K(P, P), Sj = dK(P, P);
// the transposed block has the same form with c1 and c2 swapped.  Every leaf therefore receives
//   y_leaf = dK_leaf x_leaf + dPhi_leaf S^{-1} a + Phi_leaf S^{-1} (b - Sj S^{-1} a)
// where a and b are the sums of phi and dphi of the siblings along the leaf's path to the root.
// The sums travel through the tree sweeps with 2r-long vectors [phi ; dphi].
#include <algorithm>
#include <type_traits>

#include "km_kernels.h"
#include "km_kfun.cuh"

namespace km {

// VP[leaf][col] = [Phi_leaf' x ; dPhi_leaf' x]  (nmat r values: nmat = 2, or nmat = 1 for
// Phi_leaf' x alone) for a chunk of 8 columns.  The leaf is processed in chunks of 32 rows:
// [Phi dPhi] (32 x nmat r) and x (8 x 32) are staged in shared memory as T, and thread
// q < nmat r owns output row q with 8 accumulators.  T = double (FP64 form) or ff (mixed form:
// float-pair copies of Phi and dPhi, x converted on load).
// grid (nleaf, ceil(k/8)), block 32 ceil(nmat r / 32) or 256.
constexpr int kDRows = 32;

template <typename T>
__global__ void __launch_bounds__(256) k_leaf_dphiT(const T* __restrict__ Phi, const T* __restrict__ dPhi, int r,
                                                    DTree t, const double* __restrict__ X, int64_t ldx,
                                                    double* __restrict__ VP, int k, int nmat) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int r2 = nmat * r, ldp = r2 + 1;
  T* ps = reinterpret_cast<T*>(smraw);   // kDRows x (2r + 1)
  T* xs = ps + kDRows * ldp;              // 8 x kDRows
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int c0 = blockIdx.y * 8;
  const int nc = min(8, k - c0);
  const int tid = threadIdx.x;
  T acc[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) acc[c] = T(0.0);
  for (int i0 = 0; i0 < m; i0 += kDRows) {
    const int rows = min(kDRows, m - i0);
    __syncthreads();
    for (int e = tid; e < rows * r2; e += blockDim.x) {
      const int q = e / rows, i = e - q * rows;
      ps[i * ldp + q] = q < r ? Phi[s * r + (int64_t)q * m + i0 + i] : dPhi[s * r + (int64_t)(q - r) * m + i0 + i];
    }
    for (int e = tid; e < 8 * kDRows; e += blockDim.x) {
      const int c = e / kDRows, i = e - c * kDRows;
      xs[e] = (c < nc && i < rows) ? from_double<T>(X[(int64_t)(c0 + c) * ldx + s + i0 + i]) : T(0.0);
    }
    __syncthreads();
    if (tid < r2)
      for (int i = 0; i < rows; ++i) {
        const T a = ps[i * ldp + tid];
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[c] += a * xs[c * kDRows + i];
      }
  }
  if (tid < r2)
#pragma unroll
    for (int c = 0; c < 8; ++c)
      if (c < nc) VP[(leaf * k + c0 + c) * r2 + tid] = to_double(acc[c]);
}

// Eight consecutive values from 16-byte-aligned shared memory with four 16-byte loads.
__device__ __forceinline__ void load8(const ff* p, ff (&v)[8]) {
  const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float4 f = q[k];
    v[2 * k] = ff(f.x, f.y);
    v[2 * k + 1] = ff(f.z, f.w);
  }
}
__device__ __forceinline__ void load8(const double* p, double (&v)[8]) {
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double2 d = q[k];
    v[2 * k] = d.x;
    v[2 * k + 1] = d.y;
  }
}

// y_leaf = dK_leaf x + dPhi beta1 + Phi beta2, beta1 = S^{-1} a, beta2 = S^{-1}(b - Sj beta1),
// [a ; b] = VG[leaf][col], for a chunk of 8 columns.  The betas are solved in FP64 (one warp per
// column), then x and the betas are staged in shared memory as T and each thread owns leaf rows
// with 8 accumulators, so every matrix entry read feeds 8 multiply-adds.
// grid (nleaf, ceil(k/8)), block 256.
template <typename T>
__global__ void __launch_bounds__(256) k_leaf_dnys_apply(const T* __restrict__ dKl, const T* __restrict__ Phi,
                                                         const T* __restrict__ dPhi, const double* __restrict__ Sc,
                                                         const double* __restrict__ Sj, int r, DTree t,
                                                         const double* __restrict__ X, int64_t ldx,
                                                         const double* __restrict__ VG, double* __restrict__ Y,
                                                         int64_t ldy, int k, const T* __restrict__ betas) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int c0 = blockIdx.y * 8;
  const int nc = min(8, k - c0);
  double* bd = reinterpret_cast<double*>(smraw);  // 8 x 3r : beta1 | beta2 | (spare), FP64
  T* xs = reinterpret_cast<T*>(bd + 8 * 3 * r);   // m x 8 (16-byte aligned)
  T* bs = xs + 8 * m;                              // 2r x 8 : beta1 rows, then beta2 rows
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int e = threadIdx.x; e < 8 * m; e += blockDim.x) {  // row l of the chunk at xs[8 l]
    const int c = e / m, i = e % m;
    xs[8 * i + c] = c < nc ? from_double<T>(X[(int64_t)(c0 + c) * ldx + s + i]) : T(0.0);
  }
  if (betas) {  // coefficients formed by k_dbeta
    for (int e = threadIdx.x; e < 8 * 2 * r; e += blockDim.x) {
      const int c = e / (2 * r), i = e % (2 * r);
      bs[8 * i + c] = c < nc ? betas[(leaf * k + c0 + c) * 2 * r + i] : T(0.0);
    }
  } else if (w < nc) {
    double* b1 = bd + w * 3 * r;
    double* b2 = b1 + r;
    const double* g = VG + (leaf * k + c0 + w) * 2 * r;
    for (int i = lane; i < r; i += 32) {
      b1[i] = g[i];
      b2[i] = g[r + i];
    }
    __syncwarp();
    for (int pass = 0; pass < 2; ++pass) {
      double* v = pass == 0 ? b1 : b2;
      if (pass == 1) {
        // b2 <- b2 - Sj b1
        for (int i = lane; i < r; i += 32) {
          double a = 0.0;
          for (int l = 0; l < r; ++l) a += Sj[i + (int64_t)l * r] * b1[l];
          b2[i] -= a;
        }
        __syncwarp();
      }
      // v <- S^{-1} v = Sc^{-T} Sc^{-1} v
      for (int l = 0; l < r; ++l) {
        const double vl = v[l] / Sc[(int64_t)l * r + l];
        __syncwarp();
        if (lane == 0) v[l] = vl;
        for (int i = l + 1 + lane; i < r; i += 32) v[i] -= Sc[(int64_t)l * r + i] * vl;
        __syncwarp();
      }
      for (int i = r - 1; i >= 0; --i) {
        const double vi = v[i] / Sc[(int64_t)i * r + i];
        __syncwarp();
        if (lane == 0) v[i] = vi;
        for (int l = lane; l < i; l += 32) v[l] -= Sc[i + (int64_t)l * r] * vi;
        __syncwarp();
      }
    }
    for (int i = lane; i < 2 * r; i += 32) bs[8 * i + w] = from_double<T>(b1[i]);  // row i at bs[8 i]
  } else if (w < 8) {
    for (int i = lane; i < 2 * r; i += 32) bs[8 * i + w] = T(0.0);
  }
  __syncthreads();
  const T* K = dKl + d_leaf_koff(t, leaf);
  const T* P = Phi + s * r;
  const T* dP = dPhi + s * r;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    T acc[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] = T(0.0);
    // four matrix entries are loaded ahead of their multiply-adds so that the loads overlap
    int l = 0;
    for (; l + 1 < m; l += 2) {
      const T a0 = K[i + (int64_t)l * m], a1 = K[i + (int64_t)(l + 1) * m];
      T x0[8], x1[8];
      load8(xs + 8 * l, x0);
      load8(xs + 8 * (l + 1), x1);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        acc[c] += a0 * x0[c];
        acc[c] += a1 * x1[c];
      }
    }
    for (; l < m; ++l) {
      const T a = K[i + (int64_t)l * m];
      T x0[8];
      load8(xs + 8 * l, x0);
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[c] += a * x0[c];
    }
    for (int q = 0; q < r; ++q) {
      const T dp = dP[i + (int64_t)q * m], p = P[i + (int64_t)q * m];
      T b1v[8], b2v[8];
      load8(bs + 8 * q, b1v);
      load8(bs + 8 * (r + q), b2v);
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        acc[c] += dp * b1v[c];
        acc[c] += p * b2v[c];
      }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c)
      if (c < nc) Y[(int64_t)(c0 + c) * ldy + s + i] = to_double(acc[c]);
  }
}

// C = A op(B) for r x r column-major FP64 matrices, op(B) = B or B'.  One CTA per column of C.
__global__ void k_small_gemm(const double* __restrict__ A, const double* __restrict__ B, int r, int transB,
                             double* __restrict__ Cm) {
  const int j = blockIdx.x;
  for (int i = threadIdx.x; i < r; i += blockDim.x) {
    double acc = 0.0;
    for (int l = 0; l < r; ++l) acc += A[i + (int64_t)l * r] * (transB ? B[j + (int64_t)l * r] : B[l + (int64_t)j * r]);
    Cm[i + (int64_t)j * r] = acc;
  }
}

// Landmark coefficients of the derivative products for every (leaf, column) pair p:
//   beta1 = S^{-1} a,  beta2 = S^{-1} b - M2 a,  M2 = S^{-1} Sj S^{-1},  [a ; b] = VG[p],
// the same quantities k_leaf_dnys_apply otherwise forms with triangular solves, here as
// products with the explicit r x r operators (float pairs in the mixed form).  Each CTA takes
// 8 pairs; thread q < 2r owns output row q.  Output: beta[p][0:r] = beta1, beta[p][r:2r] = beta2.
template <typename T>
__global__ void __launch_bounds__(256) k_dbeta(const T* __restrict__ Sinv, const T* __restrict__ M2, int r,
                                               const double* __restrict__ VG, int64_t npairs, T* __restrict__ beta) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* g = reinterpret_cast<T*>(smraw);  // 8 x 2r
  const int64_t p0 = (int64_t)blockIdx.x * 8;
  const int np = (int)(npairs - p0 < 8 ? npairs - p0 : 8);
  const int r2 = 2 * r;
  for (int e = threadIdx.x; e < 8 * r2; e += blockDim.x)
    g[e] = (e / r2) < np ? from_double<T>(VG[p0 * r2 + e]) : T(0.0);
  __syncthreads();
  const int q = threadIdx.x;
  if (q >= r2) return;
  const int qi = q < r ? q : q - r;
  T acc[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) acc[c] = T(0.0);
  const int boff = q < r ? 0 : r;  // S^{-1} applies to a (beta1) or to b (beta2)
  for (int l = 0; l < r; ++l) {
    const T sv = Sinv[qi + (int64_t)l * r];
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] += sv * g[c * r2 + boff + l];
  }
  if (q >= r)
    for (int l = 0; l < r; ++l) {
      const T mv = M2[qi + (int64_t)l * r];
#pragma unroll
      for (int c = 0; c < 8; ++c) acc[c] -= mv * g[c * r2 + l];
    }
#pragma unroll
  for (int c = 0; c < 8; ++c)
    if (c < np) beta[(p0 + c) * r2 + q] = acc[c];
}

// out[c] = sum_i A[i + c*lda] * B[i + c*ldb], one CTA per column (deterministic order).
__global__ void k_col_dots(const double* __restrict__ A, int64_t lda, const double* __restrict__ B, int64_t ldb,
                           int64_t n, double* __restrict__ out) {
  __shared__ double red[8];
  const int c = blockIdx.x;
  const double* a = A + (int64_t)c * lda;
  const double* b = B + (int64_t)c * ldb;
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += a[i] * b[i];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
    out[c] = s;
  }
}

// y = a x + b y over n values
__global__ void k_axpby(double* __restrict__ y, const double* __restrict__ x, double a, double b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}

// SplitMix64 finaliser (Steele, Lea and Flood, "Fast splittable pseudorandom number
// generators", OOPSLA 2014).  Probe entry (i, j) of an n x p block is +1 when the top bit of
// mix(mix(seed) + j*n + i) is set and -1 otherwise.
__device__ __forceinline__ uint64_t splitmix64_mix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void k_rademacher(double* __restrict__ out, int64_t total, uint64_t seed) {
  const uint64_t base = splitmix64_mix(seed);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = (splitmix64_mix(base + (uint64_t)e) >> 63) ? 1.0 : -1.0;
}

void launch_rademacher(double* out, int64_t n, int64_t p, uint64_t seed, cudaStream_t st) {
  const int64_t total = n * p;
  k_rademacher<<<(unsigned)std::min<int64_t>((total + 255) / 256, 4096), 256, 0, st>>>(out, total, seed);
}

void launch_axpby(double* y, const double* x, double a, double b, int64_t n, cudaStream_t st) {
  k_axpby<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(y, x, a, b, n);
}

template <typename T>
void launch_leaf_dphiT(const T* Phi, const T* dPhi, int r, const Tree& t, const double* X, int64_t ldx, double* VP,
                       int k, cudaStream_t st) {
  dim3 grid((unsigned)t.nleaf, (unsigned)((k + 7) / 8));
  const size_t sm = ((size_t)kDRows * (2 * r + 1) + 8 * kDRows) * sizeof(T);
  smem_limit((const void*)k_leaf_dphiT<T>, sm);
  k_leaf_dphiT<T><<<grid, 256, sm, st>>>(Phi, dPhi, r, dtree(t), X, ldx, VP, k, 2);
}

// VP[(leaf k + c) r + q] = Phi_leaf[:, q]' x_leaf,c: one warp per (leaf, landmark q), lanes over
// the leaf's rows (coalesced reads of Phi's column and of x), a fixed-order warp sum per
// column.  grid (nleaf, ceil(r / 8)), block 256.
template <typename T>
__global__ void __launch_bounds__(256) k_leaf_phiT(const T* __restrict__ Phi, int r, DTree t,
                                                   const double* __restrict__ X, int64_t ldx,
                                                   double* __restrict__ VP, int k) {
  const int lane = threadIdx.x & 31, q = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (q >= r) return;
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const T* pc = Phi + s * r + (int64_t)q * m;
  for (int c = 0; c < k; ++c) {
    const double* xc = X + (int64_t)c * ldx + s;
    acc_t<T> a0{}, a1{};
    int i = lane;
    for (; i + 32 < m; i += 64) {
      a0 += pc[i] * from_double<T>(xc[i]);
      a1 += pc[i + 32] * from_double<T>(xc[i + 32]);
    }
    if (i < m) a0 += pc[i] * from_double<T>(xc[i]);
    const double v = warp_sum(to_double(accv(a0) + accv(a1)));
    if (lane == 0) VP[(leaf * k + c) * r + q] = v;
  }
}

void launch_leaf_phiT(const double* Phi, int r, const Tree& t, const double* X, int64_t ldx, double* VP, int k,
                      cudaStream_t st) {
  k_leaf_phiT<double><<<dim3((unsigned)t.nleaf, (unsigned)((r + 7) / 8)), 256, 0, st>>>(Phi, r, dtree(t), X, ldx, VP,
                                                                                       k);
}

template <typename T>
void launch_leaf_dnys_apply(const T* dKl, const T* Phi, const T* dPhi, const double* Sc, const double* Sj, int r,
                            const Tree& t, const double* X, int64_t ldx, const double* VG, double* Y, int64_t ldy,
                            int k, cudaStream_t st, const T* betas) {
  dim3 grid((unsigned)t.nleaf, (unsigned)((k + 7) / 8));
  const size_t sm = (size_t)8 * 3 * r * sizeof(double) + ((size_t)8 * t.max_leaf + 8 * 2 * r) * sizeof(T);
  smem_limit((const void*)k_leaf_dnys_apply<T>, sm);
  k_leaf_dnys_apply<T><<<grid, 256, sm, st>>>(dKl, Phi, dPhi, Sc, Sj, r, dtree(t), X, ldx, VG, Y, ldy, k, betas);
}

template void launch_leaf_dphiT<double>(const double*, const double*, int, const Tree&, const double*, int64_t,
                                        double*, int, cudaStream_t);
template void launch_leaf_dphiT<ff>(const ff*, const ff*, int, const Tree&, const double*, int64_t, double*, int,
                                    cudaStream_t);
template void launch_leaf_dnys_apply<double>(const double*, const double*, const double*, const double*,
                                             const double*, int, const Tree&, const double*, int64_t,
                                             const double*, double*, int64_t, int, cudaStream_t, const double*);
template void launch_leaf_dnys_apply<ff>(const ff*, const ff*, const ff*, const double*, const double*, int,
                                         const Tree&, const double*, int64_t, const double*, double*, int64_t, int,
                                         cudaStream_t, const ff*);

// ---------------------------------------------------------------------------------------------
// Second-derivative product of the stochastic Hessian (Deriv2mul, src/HODLR/src/utils.jl:157-177)
// in the nested Nystrom form.  The landmark matrices are global, so the reference's block
// products SDBlock_mul / SDBlock_mul_t (utils.jl:110-155) are linear maps of the four projections
// [Phi' s; Phi_j' s; Phi_k' s; Phi_jk' s] of the source block onto the four expansion coefficients
// of the target block: Tmul and Tmult (R x R, R = 4r, formed once from S^{-1}, S_j, S_k, S_jk).
// A node's projections are sums of its leaves' (up-sweep, UP_SUM at width R).  The reference's
// block (a:b, c:d) of a node has the rows of its second child and the columns of its first
// (HODLRindices), so Deriv2mul adds SDBlock_mul of the first child's values to the second child
// and SDBlock_mul_t of the second child's values to the first: the down-sweep gives the second
// child Tmul (projections of the first) and the first child Tmult (projections of the second)
// on top of its parent's coefficients; a leaf then adds its dense second-derivative block and
// its four basis expansions.  Variant order: Phi, Phi_j, Phi_k,
// Phi_jk; Phi3 holds Phi_j, Phi_k, Phi_jk (n r values each, the per-leaf layout of Phi).
// ---------------------------------------------------------------------------------------------

// VP[(leaf k + c) R + v r + q] = Phi_v(leaf)' x_c.  grid (nleaf, k), block 256.
__global__ void __launch_bounds__(256) k_leaf_phi4T(const double* __restrict__ Phi, const double* __restrict__ Phi3,
                                                    int64_t nr, int r, DTree t, const double* __restrict__ X,
                                                    int64_t ldx, double* __restrict__ VP, int k) {
  extern __shared__ double xs[];  // the leaf's rows of column c
  const int64_t leaf = blockIdx.x;
  const int c = blockIdx.y;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  for (int i = threadIdx.x; i < m; i += blockDim.x) xs[i] = X[(int64_t)c * ldx + s + i];
  __syncthreads();
  const int R = 4 * r;
  for (int e = threadIdx.x; e < R; e += blockDim.x) {
    const int v = e / r, q = e - v * r;
    const double* P = (v == 0 ? Phi : Phi3 + (int64_t)(v - 1) * nr) + s * r + (int64_t)q * m;
    double acc = 0.0;
    for (int i = 0; i < m; ++i) acc += P[i] * xs[i];
    VP[(leaf * k + c) * R + e] = acc;
  }
}

// Down-sweep of one level: VG(child 1) = g + Tmult VP(child 2), VG(child 2) = g + Tmul VP(child 1),
// g the parent's coefficients (zero at the root).  Tmul, Tmult column-major R x R.
// grid (nodes at the level, k), block 256.
__global__ void __launch_bounds__(256) k_d2_down(const double* __restrict__ Tmul, const double* __restrict__ Tmult,
                                                 int R, int top, int64_t cslot0, int64_t nslot0,
                                                 const double* __restrict__ VP, double* __restrict__ VG, int k) {
  extern __shared__ double sd[];  // g, p1, p2 (R each)
  double* g = sd;
  double* p1 = g + R;
  double* p2 = p1 + R;
  const int64_t kk = blockIdx.x;
  const int c = blockIdx.y;
  const int64_t s1 = cslot0 + 2 * kk, s2 = s1 + 1;
  for (int e = threadIdx.x; e < R; e += blockDim.x) {
    g[e] = top ? 0.0 : VG[((nslot0 + kk) * k + c) * R + e];
    p1[e] = VP[(s1 * k + c) * R + e];
    p2[e] = VP[(s2 * k + c) * R + e];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < R; e += blockDim.x) {
    double a1 = g[e], a2 = g[e];
    for (int f = 0; f < R; ++f) {
      a1 += Tmult[e + (int64_t)f * R] * p2[f];
      a2 += Tmul[e + (int64_t)f * R] * p1[f];
    }
    VG[(s1 * k + c) * R + e] = a1;
    VG[(s2 * k + c) * R + e] = a2;
  }
}

// Y_leaf = D2_leaf x_leaf + sum_v Phi_v(leaf) G_v(leaf); G = 0 when VG is null (one leaf).
// grid (nleaf, k), block 256; D2 the dense leaf blocks (column-major m x m at the leaf offset).
__global__ void __launch_bounds__(256) k_leaf_d2_apply(const double* __restrict__ D2, const double* __restrict__ Phi,
                                                       const double* __restrict__ Phi3, int64_t nr, int r, DTree t,
                                                       const double* __restrict__ X, int64_t ldx,
                                                       const double* __restrict__ VG, double* __restrict__ Y,
                                                       int64_t ldy, int k) {
  extern __shared__ double sa[];  // x (m), G (4r)
  const int64_t leaf = blockIdx.x;
  const int c = blockIdx.y;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int R = 4 * r;
  double* xs = sa;
  double* G = sa + m;
  for (int i = threadIdx.x; i < m; i += blockDim.x) xs[i] = X[(int64_t)c * ldx + s + i];
  for (int e = threadIdx.x; e < R; e += blockDim.x) G[e] = VG ? VG[(leaf * k + c) * R + e] : 0.0;
  __syncthreads();
  const double* A = D2 + d_leaf_koff(t, leaf);
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < m; ++j) acc += A[(int64_t)j * m + i] * xs[j];
    for (int v = 0; v < 4; ++v) {
      const double* P = (v == 0 ? Phi : Phi3 + (int64_t)(v - 1) * nr) + s * r;
      for (int q = 0; q < r; ++q) acc += P[(int64_t)q * m + i] * G[v * r + q];
    }
    Y[(int64_t)c * ldy + s + i] = acc;
  }
}

// Tmul and Tmult (column-major R x R) from M = [A, Bj, Bk, Bjk, Cjk, Ckj] (r x r each), with
// A = S^{-1}, B_x = A S_x A, Cjk = Bj Sk A, Ckj = Bk Sj A; blocks (output variant, input variant):
//   Tmul  = [[-Ckj + Bjk - Cjk - Bk, Bj, 0, A], [-Bk, 0, A, 0], [Bj + A, 0, 0, 0], [A, 0, 0, 0]]
//   Tmult = [[-Cjk + Bjk - Ckj, -Bk, Bj, A], [-Bk, 0, A, 0], [Bj, 0, A, 0], [A, 0, 0, 0]]
// (SDBlock_mul and SDBlock_mul_t read term by term as maps of the four projections).
__global__ void k_d2_assemble(const double* __restrict__ M, int r, double* __restrict__ Tmul,
                              double* __restrict__ Tmult) {
  const int R = 4 * r;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)R * R) return;
  const int row = (int)(e % R), col = (int)(e / R);
  const int bi = row / r, bj = col / r;
  const int64_t rr = (int64_t)r * r;
  const int64_t o = (row - bi * r) + (int64_t)(col - bj * r) * r;
  const double A = M[o], Bj = M[rr + o], Bk = M[2 * rr + o], Bjk = M[3 * rr + o], Cjk = M[4 * rr + o],
               Ckj = M[5 * rr + o];
  double u = 0.0, w = 0.0;
  if (bi == 0) {
    if (bj == 0) {
      u = -Ckj + Bjk - Cjk - Bk;
      w = -Cjk + Bjk - Ckj;
    } else if (bj == 1) {
      u = Bj;
      w = -Bk;
    } else if (bj == 2) {
      w = Bj;
    } else {
      u = A;
      w = A;
    }
  } else if (bi == 1) {
    if (bj == 0) {
      u = -Bk;
      w = -Bk;
    } else if (bj == 2) {
      u = A;
      w = A;
    }
  } else if (bi == 2) {
    if (bj == 0) {
      u = Bj + A;
      w = Bj;
    } else if (bj == 2) {
      w = A;
    }
  } else if (bj == 0) {
    u = A;
    w = A;
  }
  Tmul[e] = u;
  Tmult[e] = w;
}

void launch_leaf_phi4T(const double* Phi, const double* Phi3, int r, const Tree& t, const double* X, int64_t ldx,
                       double* VP, int k, cudaStream_t st) {
  const size_t sm = (size_t)t.max_leaf * sizeof(double);
  smem_limit((const void*)k_leaf_phi4T, sm);
  k_leaf_phi4T<<<dim3((unsigned)t.nleaf, (unsigned)k), 256, sm, st>>>(Phi, Phi3, t.n * (int64_t)r, r, dtree(t), X,
                                                                      ldx, VP, k);
}

void launch_d2_down(const double* Tmul, const double* Tmult, int r, const Tree& t, int level, const double* VP,
                    double* VG, int k, cudaStream_t st) {
  const int R = 4 * r;
  const int64_t cslot0 = level == 1 ? 0 : t.nleaf + t.node_off[level - 1];
  const int64_t nslot0 = t.nleaf + t.node_off[level];
  const size_t sm = (size_t)3 * R * sizeof(double);
  smem_limit((const void*)k_d2_down, sm);
  k_d2_down<<<dim3((unsigned)t.nodes_at(level), (unsigned)k), 256, sm, st>>>(Tmul, Tmult, R, level >= t.L ? 1 : 0,
                                                                             cslot0, nslot0, VP, VG, k);
}

void launch_leaf_d2_apply(const double* D2, const double* Phi, const double* Phi3, int r, const Tree& t,
                          const double* X, int64_t ldx, const double* VG, double* Y, int64_t ldy, int k,
                          cudaStream_t st) {
  const size_t sm = ((size_t)t.max_leaf + 4 * r) * sizeof(double);
  smem_limit((const void*)k_leaf_d2_apply, sm);
  k_leaf_d2_apply<<<dim3((unsigned)t.nleaf, (unsigned)k), 256, sm, st>>>(D2, Phi, Phi3, t.n * (int64_t)r, r,
                                                                         dtree(t), X, ldx, VG, Y, ldy, k);
}

void launch_d2_assemble(const double* M, int r, double* Tmul, double* Tmult, cudaStream_t st) {
  const int64_t tot = (int64_t)16 * r * r;
  k_d2_assemble<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(M, r, Tmul, Tmult);
}

// ---------------------------------------------------------------------------------------------
// Trace form of the stochastic gradient.  The gradient needs only the weighted sum over the
// columns x_c of X = [T alpha] of x_c' dK_j x_c (w_c = 1/p for the probes; wa = -1, or
// -n / y'alpha for the profile likelihood, for alpha), never dK_j x_c itself.  Every
// off-diagonal block of the Nystrom HODLR is Phi_c2 S^{-1} Phi_c1' with the one landmark set
// (nystrom_uvt, src/factorizations.jl:86-94), so the matrix is
//   K_H = Phi S^{-1} Phi' + sum_leaves (K_l - Phi_l S^{-1} Phi_l'),
// and with A = Phi' x and B_j = dPhi_j' x for the whole vector, phi_l and dphi_l for leaf l,
//   x' dK_j x = q_j(A, B_j) + sum_l [ x_l' dK_j,l x_l - q_j(phi_l, dphi_l) ],
//   q_j(u, v) = 2 u~' v - u~' Sj u~,   u~ = S^{-1} u,   Sj = dK_j(P, P),
// the same quantity as the reference's per-probe products summed over the probes
// (stochasticgradient.jl:14-26).  Leaf terms: sum_c w_c x_l,c' dK_j,l x_l,c = <dK_j,l, G_l>,
// with the leaf Gram matrix G_l formed tile by tile in registers and the three derivatives
// evaluated on the fly (k_leaf_dk_gram); landmark terms: the projections [phi ; dphi_0 ;
// dphi_1 ; dphi_2] of every (leaf, column) pair (k_leaf_proj3, k_nugget_proj), their sums over the leaves
// (k_proj_total) and the weighted quadratic forms (k_landmark).  No dK leaf, Gram matrix or
// tree sweep is stored.
// ---------------------------------------------------------------------------------------------

// dPhi2[j n r + s r + c m + i] = dK_j(x_{s+i}, p_c) for the scale and range parameters j = 0, 1
// (the panel layout of Phi, two panels), float pairs in the mixed form.  The nugget derivative
// [x == p] is handled by k_nugget_proj.  grid (ceil(m r / 256), nleaf), block 256.
template <typename T>
__global__ void k_eval_dphi2(const double* __restrict__ pts, const double* __restrict__ lnd,
                             const float* __restrict__ P3, const float* __restrict__ L3, int r, DTree t,
                             KParams kp, T* __restrict__ dPhi2) {
  extern __shared__ double sl[];  // 2r
  for (int q = threadIdx.x; q < 2 * r; q += blockDim.x) sl[q] = lnd[q];
  __syncthreads();
  const int64_t leaf = blockIdx.y;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)m * r) return;
  const int c = (int)(e / m), i = (int)(e % m);
  const double x = pts[2 * (s + i)], y = pts[2 * (s + i) + 1];
  const int64_t o = s * r + (int64_t)c * m + i, nr = t.n * (int64_t)r;
  if constexpr (std::is_same<T, ff>::value) {
    f3 x1, y1, x2, y2;
    load_p3(P3, s + i, x1, y1);
    load_p3(L3, c, x2, y2);
    ff v[3];
    dkernel3_ffp(kp, x1, y1, x2, y2, v);
    dPhi2[o] = v[0];
    dPhi2[o + nr] = v[1];
  } else {
    double v[3];
    dkernel3(kp, x, y, sl[2 * c], sl[2 * c + 1], v);
    dPhi2[o] = v[0];
    dPhi2[o + nr] = v[1];
  }
}

// VP[(leaf k + c) W + mat r + q] = sum_i A_mat[i][q] X[i][c]: the projections phi = Phi_l' x_c,
// dphi_0 = dPhi_0,l' x_c and dphi_1 = dPhi_1,l' x_c (W = 4r; the nugget block mat = 3 comes from
// k_nugget_proj), one small GEMM per (leaf, matrix), register-tiled.  A CTA takes the r rows of
// matrix mat = blockIdx.y and 8g columns (g <= 10); thread (u, v) = (tid % uq, tid / uq),
// uq = ceil(r / 4), accumulates the 4 x 8 block q = u + uq a, c = c0 + v + g b (strided, so that
// the shared-memory reads of a warp fall in distinct banks).  The leaf rows go in chunks of 32:
// A_mat (r x 32) and X (8g x 32) are staged in shared memory as T along i with a padded stride;
// rows past the leaf are zeros.  grid (nleaf, 3, ceil(k / 8g)), block uq g.
constexpr int kPjK = 32, kPjS = kPjK + 1, kPjMaxG = 10, kPjMaxU = (kMaxNysRank + 3) / 4;

template <typename T>
__global__ void __launch_bounds__(kPjMaxU * kPjMaxG, 2)
    k_leaf_proj3(const T* __restrict__ Phi, const T* __restrict__ dPhi2, int r, DTree t, const T* __restrict__ X,
                 int64_t ldx, double* __restrict__ VP, int k, int g) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int uq = (r + 3) / 4;
  T* As = reinterpret_cast<T*>(smraw);  // 4 uq x kPjS, [q][i]
  T* Xs = As + 4 * uq * kPjS;           // 8g x kPjS, [c][i]
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int mat = blockIdx.y;
  const T* A = (mat == 0 ? Phi : dPhi2 + (int64_t)(mat - 1) * t.n * r) + s * r;
  const int W = 4 * r;
  const int c0 = blockIdx.z * 8 * g;
  const int ncol = min(8 * g, k - c0);
  const int tid = threadIdx.x, nth = blockDim.x;
  const int u = tid % uq, v = tid / uq;
  acc_t<T> acc[4][8] = {};
  for (int i0 = 0; i0 < m; i0 += kPjK) {
    const int rows = min(kPjK, m - i0);
    __syncthreads();
    for (int e = tid; e < 4 * uq * kPjK; e += nth) {
      const int q = e / kPjK, i = e - q * kPjK;
      As[q * kPjS + i] = (q < r && i < rows) ? A[(int64_t)q * m + i0 + i] : T(0.0);
    }
    for (int e = tid; e < 8 * g * kPjK; e += nth) {
      const int cl = e / kPjK, i = e - cl * kPjK;
      Xs[cl * kPjS + i] = (cl < ncol && i < rows) ? X[(int64_t)(c0 + cl) * ldx + s + i0 + i] : T(0.0);
    }
    __syncthreads();
#pragma unroll 2
    for (int i = 0; i < kPjK; ++i) {
      T av[4], xv[8];
#pragma unroll
      for (int a = 0; a < 4; ++a) av[a] = As[(u + uq * a) * kPjS + i];
#pragma unroll
      for (int b = 0; b < 8; ++b) xv[b] = Xs[(v + g * b) * kPjS + i];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] += av[a] * xv[b];
    }
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const int q = u + uq * a, cl = v + g * b;
      if (q < r && cl < ncol) VP[(leaf * k + c0 + cl) * W + mat * r + q] = to_double(accv(acc[a][b]));
    }
}

// VP[(leaf k + c) W + 3r + q] = sum over the leaf's points x_i equal to landmark p_q (coordinate by
// coordinate) of X[i][c]: the projection on the nugget derivative dK_2(X, P) = [x == p], a
// 0/1 matrix with at most one entry per row for distinct points.  Thread q scans the leaf once;
// a landmark with several equal points (repeated points) rescans it per column, in order.
// grid nleaf, block 32 ceil(r / 32).
__global__ void k_nugget_proj(const double* __restrict__ pts, const double* __restrict__ lnd, int r, DTree t,
                              const double* __restrict__ X, int64_t ldx, double* __restrict__ VP, int k) {
  const int q = threadIdx.x;
  if (q >= r) return;
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int W = 4 * r;
  const double px = lnd[2 * q], py = lnd[2 * q + 1];
  int first = -1, cnt = 0;
  for (int i = 0; i < m; ++i)
    if (pts[2 * (s + i)] == px && pts[2 * (s + i) + 1] == py) {
      if (first < 0) first = i;
      ++cnt;
    }
  for (int c = 0; c < k; ++c) {
    double v = 0.0;
    if (cnt == 1) {
      v = X[(int64_t)c * ldx + s + first];
    } else if (cnt > 1) {
      for (int i = first; i < m; ++i)
        if (pts[2 * (s + i)] == px && pts[2 * (s + i) + 1] == py) v += X[(int64_t)c * ldx + s + i];
    }
    VP[(leaf * k + c) * W + 3 * r + q] = v;
  }
}

// VP[(nleaf k + c) W + q] = sum over the leaves of VP[(leaf k + c) W + q]: A and B_j of the
// whole vector, in a fixed order (warp w sums the leaves w, w + 8, ..., then the eight warp sums
// are added in order).  grid (k, ceil(W / 32)), block 256.
__global__ void k_proj_total(double* __restrict__ VP, int W, int64_t nleaf, int k) {
  __shared__ double red[8][32];
  const int c = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int q = blockIdx.y * 32 + lane;
  double s = 0.0;
  if (q < W) {
#pragma unroll 4
    for (int64_t l = w; l < nleaf; l += 8) s += VP[(l * k + c) * W + q];
  }
  red[w][lane] = s;
  __syncthreads();
  if (w == 0 && q < W) {
    double tot = 0.0;
#pragma unroll
    for (int u = 0; u < 8; ++u) tot += red[u][lane];
    VP[(nleaf * k + c) * W + q] = tot;
  }
}

// Weighted quadratic forms of one leaf (blockIdx.x < nleaf, sign -1) or of the whole vector
// (blockIdx.x = nleaf: the sums of k_proj_total, sign +1):
//   part[j (nleaf + 1) + l] = sign * sum_c w_c q_j(u_c, v_j,c) = sign * (2 D_j - <Sj, H>),
//   D_j = sum_c w_c u~_c' v_j,c,  H = sum_c w_c u~_c u~_c',  u~ = S^{-1} u,
// with u = VP[.. + 0 : r] and v_j = VP[.. + (j + 1) r : (j + 2) r].  Columns go in chunks of 16:
// the chunk's projections (W x 16) and S^{-1} are staged in shared memory as T; thread
// (cc = tid % 16, g = tid / 16) forms u~ for the rows g, g + 16, ... of column cc, and each thread
// keeps up to 13 entries of the packed lower triangle of H (r <= 80) in registers.
// grid nleaf + 1, block 256.
constexpr int kLmCols = 16;
constexpr int kLmS = kLmCols + 2;  // padded row stride of u~: the rows of a quarter warp start in distinct banks
constexpr int kLmH = (kMaxNysRank * (kMaxNysRank + 1) / 2 + 255) / 256;

template <typename T>
__global__ void __launch_bounds__(256) k_landmark(const double* __restrict__ VP, int r, int k, int p, double wa,
                                                  const T* __restrict__ Sinv, const T* __restrict__ Sj3,
                                                  int64_t nleaf, double* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int W = 4 * r, rr = r * r;
  T* si = reinterpret_cast<T*>(smraw);  // r x r, S^{-1} (column-major), padded to an even count
  T* vs = si + ((rr + 1) & ~1);         // W x 16, [q][cc] (16-byte aligned for load8)
  T* ut = vs + W * kLmCols;             // r x 16 (row stride kLmS), u~
  T* uw = ut + r * kLmS;                // r x 16 (row stride kLmS), w_c u~
  __shared__ double red[8][6];
  const int64_t l = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, wp = tid >> 5;
  const int cc = tid & (kLmCols - 1), g = tid / kLmCols;
  const int nh = r * (r + 1) / 2;
  for (int e = tid; e < rr; e += blockDim.x) si[e] = Sinv[e];
  // the entries of H this thread owns: e = tid + 256 u, (i, a) with i >= a, packed by columns
  int hi[kLmH], ha[kLmH];
#pragma unroll
  for (int u = 0; u < kLmH; ++u) {
    int e = tid + 256 * u, a = 0;
    if (e < nh) {
      while (e >= r - a) {
        e -= r - a;
        ++a;
      }
      hi[u] = a + e;
      ha[u] = a;
    } else {
      hi[u] = ha[u] = 0;
    }
  }
  acc_t<T> h[kLmH] = {};
  acc_t<T> d[3] = {};
  for (int c0 = 0; c0 < k; c0 += kLmCols) {
    const int nc = min(kLmCols, k - c0);
    __syncthreads();
    for (int e = tid; e < W * kLmCols; e += blockDim.x) {
      const int c = e / W, q = e - c * W;
      vs[q * kLmCols + c] = c < nc ? from_double<T>(VP[(l * k + c0 + c) * W + q]) : T(0.0);
    }
    __syncthreads();
    const int col = c0 + cc;
    const T w = cc < nc ? from_double<T>(col < p ? 1.0 / (double)p : wa) : T(0.0);
    for (int i = g; i < r; i += 256 / kLmCols) {
      acc_t<T> a{};
      for (int q = 0; q < r; ++q) a += si[i + q * r] * vs[q * kLmCols + cc];
      const T v = accv(a);
      const T vw = T(v * w);
      ut[i * kLmS + cc] = v;
      uw[i * kLmS + cc] = vw;
#pragma unroll
      for (int j = 0; j < 3; ++j) d[j] += vw * vs[((j + 1) * r + i) * kLmCols + cc];
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kLmH; ++u)
      if (tid + 256 * u < nh) {
#pragma unroll
        for (int q0 = 0; q0 < kLmCols; q0 += 8) {
          T x[8], y[8];
          load8(uw + hi[u] * kLmS + q0, x);
          load8(ut + ha[u] * kLmS + q0, y);
#pragma unroll
          for (int q = 0; q < 8; ++q) h[u] += x[q] * y[q];
        }
      }
  }
  // <Sj, H>: off-diagonal entries twice (Sj and H symmetric)
  double v[6];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    v[j] = to_double(accv(d[j]));
    double qj = 0.0;
#pragma unroll
    for (int u = 0; u < kLmH; ++u)
      if (tid + 256 * u < nh) {
        const double hv = to_double(accv(h[u])) * (hi[u] == ha[u] ? 1.0 : 2.0);
        qj += to_double(Sj3[(int64_t)j * rr + hi[u] + (int64_t)ha[u] * r]) * hv;
      }
    v[3 + j] = qj;
  }
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double sv = warp_sum(v[j]);
    if (lane == 0) red[wp][j] = sv;
  }
  __syncthreads();
  if (tid < 3) {
    double dj = 0.0, qj = 0.0;
    for (int u = 0; u < 8; ++u) {
      dj += red[u][tid];
      qj += red[u][3 + tid];
    }
    const double sign = l == nleaf ? 1.0 : -1.0;
    part[tid * (nleaf + 1) + l] = sign * (2.0 * dj - qj);
  }
}

__device__ __forceinline__ double twice(double x) { return x + x; }
__device__ __forceinline__ ff twice(ff x) { return ff(x.hi + x.hi, x.lo + x.lo); }

// part[j nleaf S + leaf S + z] = part z < S of <dK_j,leaf, G_leaf> for the three parameters, G_leaf = sum_{c < p} x_c x_c'
// / p + wa x_p x_p' over the columns of X (n x (p + 1), leading dimension n; double, or float
// pairs for the mixed form).  CTA (leaf, z) walks the lower-triangle 32 x 32 tiles z, z + S, ... of
// its leaf (numbered row by row): the tile
// of G from 32-column chunks of X staged in shared memory (thread (tx, ty) takes rows tx and
// columns ty + 8 q), the derivative entries evaluated in registers (dkernel3 / dkernel3_ff, one
// distance and one exponential for the three), off-diagonal entries counted twice.
// grid (nleaf, S), block (32, 8).
template <typename T>
__global__ void __launch_bounds__(256) k_leaf_dk_gram(const double* __restrict__ pts, const float* __restrict__ P3,
                                                      KParams kp,
                                                      const T* __restrict__ X, int64_t n, int p, double wa,
                                                      DTree t, double* __restrict__ part) {
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int nt = (m + 31) / 32;
  __shared__ T xr[32][33];
  __shared__ T xc[32][33];
  __shared__ double red[8][3];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
  const T wp = from_double<T>(p > 0 ? 1.0 / (double)p : 0.0), w_a = from_double<T>(wa);
  acc_t<T> tot[3] = {};
  const int z = blockIdx.y, S = gridDim.y;
  int ti = 0, tj = z;  // tile number z: row ti, column tj <= ti
  while (tj > ti) {
    tj -= ti + 1;
    ++ti;
  }
  for (; ti < nt;) {
    {
      const int i = ti * 32 + tx;
      acc_t<T> sp[4] = {}, sa[4] = {};
      for (int c0 = 0; c0 <= p; c0 += 32) {
        __syncthreads();
        for (int e = tid; e < 32 * 32; e += 256) {
          const int cq = e >> 5, rq = e & 31;  // column cq of the chunk, row rq of the tile
          const int c = c0 + cq;
          const int ri = ti * 32 + rq, rj = tj * 32 + rq;
          xr[rq][cq] = (c <= p && ri < m) ? X[(int64_t)c * n + s + ri] : T(0.0);
          xc[rq][cq] = (c <= p && rj < m) ? X[(int64_t)c * n + s + rj] : T(0.0);
        }
        __syncthreads();
        const int cend = min(32, p - c0);  // probe columns of this chunk; column p (alpha) apart
        for (int cq = 0; cq < cend; ++cq) {
          const T a = xr[tx][cq];
#pragma unroll
          for (int q = 0; q < 4; ++q) sp[q] += a * xc[ty + 8 * q][cq];
        }
        if (p - c0 < 32) {
          const T a = xr[tx][p - c0];
#pragma unroll
          for (int q = 0; q < 4; ++q) sa[q] += a * xc[ty + 8 * q][p - c0];
        }
      }
      double xi = 0.0, yi = 0.0;
      f3 x3i{}, y3i{};
      if (i < m) {
        if constexpr (std::is_same<T, ff>::value) {
          load_p3(P3, s + i, x3i, y3i);
        } else {
          xi = pts[2 * (s + i)];
          yi = pts[2 * (s + i) + 1];
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int a = tj * 32 + ty + 8 * q;
        if (i < m && a < m && i >= a) {
          T gv = T(accv(sp[q]) * wp) + T(accv(sa[q]) * w_a);
          if (i > a) gv = twice(gv);
          if constexpr (std::is_same<T, ff>::value) {
            f3 x3a, y3a;
            load_p3(P3, s + a, x3a, y3a);
            ff dk[3];
            dkernel3_ffp(kp, x3i, y3i, x3a, y3a, dk);
#pragma unroll
            for (int j = 0; j < 3; ++j) tot[j] += gv * dk[j];
          } else {
            const double xa = pts[2 * (s + a)], ya = pts[2 * (s + a) + 1];
            double dk[3];
            dkernel3(kp, xi, yi, xa, ya, dk);
#pragma unroll
            for (int j = 0; j < 3; ++j) tot[j] += gv * dk[j];
          }
        }
      }
    }
    tj += S;  // the next tile of this part
    while (tj > ti) {
      tj -= ti + 1;
      ++ti;
    }
  }
  double v[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    v[j] = warp_sum(to_double(accv(tot[j])));
    if (tx == 0) red[ty][j] = v[j];
  }
  __syncthreads();
  if (tid < 3) {
    double sum = 0.0;
    for (int u = 0; u < 8; ++u) sum += red[u][tid];
    part[(int64_t)tid * t.nleaf * S + leaf * S + z] = sum;
  }
}

// out[j] = scale (sum_q a[j na + q] + sum_q b[j nb + q]), j < 3: thread tid adds the entries tid,
// tid + 256, ... in order, then the 256 sums are added by a fixed tree.  grid 3, block 256.
__global__ void k_grad_final(const double* __restrict__ a, int64_t na, const double* __restrict__ b, int64_t nb,
                             double scale, double* __restrict__ out) {
  __shared__ double red[256];
  const int j = blockIdx.x, tid = threadIdx.x;
  double s = 0.0;
  for (int64_t q = tid; q < na; q += 256) s += a[j * na + q];
  for (int64_t q = tid; q < nb; q += 256) s += b[j * nb + q];
  red[tid] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (tid < o) red[tid] += red[tid + o];
    __syncthreads();
  }
  if (tid == 0) out[j] = scale * red[0];
}

template <typename T>
void launch_eval_dphi2(const double* pts, const double* lnd, const float* P3, const float* L3, int r, const Tree& t,
                       KParams kp, T* dPhi2, cudaStream_t st) {
  dim3 grid((unsigned)((t.max_leaf * r + 255) / 256), (unsigned)t.nleaf);
  k_eval_dphi2<T><<<grid, 256, 2 * r * sizeof(double), st>>>(pts, lnd, P3, L3, r, dtree(t), kp, dPhi2);
}

template <typename T>
void launch_leaf_proj3(const T* Phi, const T* dPhi2, int r, const Tree& t, const T* X, int64_t ldx, double* VP, int k,
                       cudaStream_t st) {
  const int g = std::min(kPjMaxG, (k + 7) / 8), uq = (r + 3) / 4;
  dim3 grid((unsigned)t.nleaf, 3u, (unsigned)((k + 8 * g - 1) / (8 * g)));
  const size_t sm = (size_t)(4 * uq + 8 * g) * kPjS * sizeof(T);
  smem_limit((const void*)k_leaf_proj3<T>, sm);
  k_leaf_proj3<T><<<grid, uq * g, sm, st>>>(Phi, dPhi2, r, dtree(t), X, ldx, VP, k, g);
}

void launch_nugget_proj(const double* pts, const double* lnd, int r, const Tree& t, const double* X, int64_t ldx,
                        double* VP, int k, cudaStream_t st) {
  k_nugget_proj<<<(unsigned)t.nleaf, 32 * ((r + 31) / 32), 0, st>>>(pts, lnd, r, dtree(t), X, ldx, VP, k);
}

void launch_proj_total(double* VP, int W, int64_t nleaf, int k, cudaStream_t st) {
  k_proj_total<<<dim3((unsigned)k, (unsigned)((W + 31) / 32)), 256, 0, st>>>(VP, W, nleaf, k);
}

template <typename T>
void launch_landmark(const double* VP, int r, int k, int p, double wa, const T* Sinv, const T* Sj3, int64_t nleaf,
                     double* part, cudaStream_t st) {
  const size_t sm = (size_t)(((r * r + 1) & ~1) + 4 * r * kLmCols + 2 * r * kLmS) * sizeof(T);
  smem_limit((const void*)k_landmark<T>, sm);
  k_landmark<T><<<(unsigned)(nleaf + 1), 256, sm, st>>>(VP, r, k, p, wa, Sinv, Sj3, nleaf, part);
}

int leaf_dk_gram_parts(const Tree& t) {
  const int nt = (int)((t.max_leaf + 31) / 32);
  return (int)std::max<int64_t>(1, std::min<int64_t>(nt * (nt + 1) / 2, 4096 / std::max<int64_t>(t.nleaf, 1)));
}

template <typename T>
void launch_leaf_dk_gram(const double* pts, const float* P3, KParams kp, const T* X, int64_t n, int p, double wa,
                         const Tree& t, double* part, cudaStream_t st) {
  const int S = leaf_dk_gram_parts(t);
  k_leaf_dk_gram<T><<<dim3((unsigned)t.nleaf, (unsigned)S), dim3(32, 8), 0, st>>>(pts, P3, kp, X, n, p, wa,
                                                                                  dtree(t), part);
}

void launch_grad_final(const double* a, int64_t na, const double* b, int64_t nb, double scale, double* out,
                       cudaStream_t st) {
  k_grad_final<<<3, 256, 0, st>>>(a, na, b, nb, scale, out);
}

template void launch_eval_dphi2<double>(const double*, const double*, const float*, const float*, int, const Tree&,
                                        KParams, double*, cudaStream_t);
template void launch_eval_dphi2<ff>(const double*, const double*, const float*, const float*, int, const Tree&,
                                    KParams, ff*, cudaStream_t);
template void launch_leaf_proj3<double>(const double*, const double*, int, const Tree&, const double*, int64_t,
                                        double*, int, cudaStream_t);
template void launch_leaf_proj3<ff>(const ff*, const ff*, int, const Tree&, const ff*, int64_t, double*, int,
                                    cudaStream_t);
template void launch_landmark<double>(const double*, int, int, int, double, const double*, const double*, int64_t,
                                      double*, cudaStream_t);
template void launch_landmark<ff>(const double*, int, int, int, double, const ff*, const ff*, int64_t, double*,
                                  cudaStream_t);
template void launch_leaf_dk_gram<double>(const double*, const float*, KParams, const double*, int64_t, int, double,
                                          const Tree&, double*, cudaStream_t);
template void launch_leaf_dk_gram<ff>(const double*, const float*, KParams, const ff*, int64_t, int, double,
                                      const Tree&, double*, cudaStream_t);

void launch_small_gemm(const double* A, const double* B, int r, int transB, double* C, cudaStream_t st) {
  k_small_gemm<<<r, 128, 0, st>>>(A, B, r, transB, C);
}

template <typename T>
void launch_dbeta(const T* Sinv, const T* M2, int r, const double* VG, int64_t npairs, T* beta, cudaStream_t st) {
  if (npairs <= 0) return;
  const size_t sm = (size_t)8 * 2 * r * sizeof(T);
  k_dbeta<T><<<(unsigned)((npairs + 7) / 8), 256, sm, st>>>(Sinv, M2, r, VG, npairs, beta);
}
template void launch_dbeta<ff>(const ff*, const ff*, int, const double*, int64_t, ff*, cudaStream_t);
template void launch_dbeta<double>(const double*, const double*, int, const double*, int64_t, double*, cudaStream_t);

void launch_col_dots(const double* A, int64_t lda, const double* B, int64_t ldb, int64_t n, int k,
                     double* out, cudaStream_t st) {
  k_col_dots<<<k, 256, 0, st>>>(A, lda, B, ldb, n, out);
}

}  // namespace km
