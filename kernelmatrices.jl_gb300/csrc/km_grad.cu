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

#include "km_kernels.h"

namespace km {

// VP[leaf][col] = [Phi_leaf' x ; dPhi_leaf' x]  (2r values).  grid (nleaf, ceil(k/8)), block 256.
__global__ void __launch_bounds__(256) k_leaf_dphiT(const double* __restrict__ Phi, const double* __restrict__ dPhi,
                                                    int r, DTree t, const double* __restrict__ X, int64_t ldx,
                                                    double* __restrict__ VP, int k) {
  extern __shared__ double sm[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int col = blockIdx.y * 8 + w;
  if (col >= k) return;
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  double* x = sm + (size_t)w * m;
  const double* src = X + (int64_t)col * ldx + s;
  for (int i = lane; i < m; i += 32) x[i] = src[i];
  __syncwarp();
  double* out = VP + (leaf * k + col) * 2 * r;
  for (int c = 0; c < 2 * r; ++c) {
    const double* pc = (c < r ? Phi + s * r + (int64_t)c * m : dPhi + s * r + (int64_t)(c - r) * m);
    double acc = 0.0;
    for (int i = lane; i < m; i += 32) acc += pc[i] * x[i];
    acc = warp_sum(acc);
    if (lane == 0) out[c] = acc;
  }
}

// y_leaf = dK_leaf x + dPhi beta1 + Phi beta2, beta1 = S^{-1} a, beta2 = S^{-1}(b - Sj beta1),
// [a ; b] = VG[leaf][col].  grid (nleaf, ceil(k/8)), block 256.
__global__ void __launch_bounds__(256) k_leaf_dnys_apply(const double* __restrict__ dKl, const double* __restrict__ Phi,
                                                         const double* __restrict__ dPhi, const double* __restrict__ Sc,
                                                         const double* __restrict__ Sj, int r, DTree t,
                                                         const double* __restrict__ X, int64_t ldx,
                                                         const double* __restrict__ VG, double* __restrict__ Y,
                                                         int64_t ldy, int k) {
  extern __shared__ double sm[];
  const int64_t leaf = blockIdx.x;
  const int m = d_leaf_size(t, leaf);
  const int64_t s = d_leaf_start(t, leaf);
  const int c0 = blockIdx.y * 8;
  const int nc = min(8, k - c0);
  double* xs = sm;            // 8 x m
  double* bs = sm + 8 * m;    // 8 x 3r : beta1 | beta2 | tmp
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int e = threadIdx.x; e < nc * m; e += blockDim.x) {
    const int c = e / m, i = e % m;
    xs[c * m + i] = X[(int64_t)(c0 + c) * ldx + s + i];
  }
  if (w < nc) {
    double* b1 = bs + w * 3 * r;
    double* b2 = b1 + r;
    const double* g = VG + (leaf * k + c0 + w) * 2 * r;
    for (int i = lane; i < r; i += 32) {
      b1[i] = g[i];
      b2[i] = g[r + i];
    }
    __syncwarp();
    // b1 <- S^{-1} b1 = Sc^{-T} Sc^{-1} b1
    for (int pass = 0; pass < 2; ++pass) {
      double* v = pass == 0 ? b1 : b2;
      if (pass == 1) {
        // b2 <- b2 - Sj b1
        for (int i = lane; i < r; i += 32) {
          double acc = 0.0;
          for (int l = 0; l < r; ++l) acc += Sj[i + (int64_t)l * r] * b1[l];
          b2[i] -= acc;
        }
        __syncwarp();
      }
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
  }
  __syncthreads();
  const double* K = dKl + d_leaf_koff(t, leaf);
  const double* P = Phi + s * r;
  const double* dP = dPhi + s * r;
  for (int e = threadIdx.x; e < nc * m; e += blockDim.x) {
    const int c = e / m, i = e % m;
    const double* xc = xs + c * m;
    double acc = 0.0;
    for (int l = 0; l < m; ++l) acc += K[i + (int64_t)l * m] * xc[l];
    const double* b1 = bs + c * 3 * r;
    const double* b2 = b1 + r;
    for (int q = 0; q < r; ++q) acc += dP[i + (int64_t)q * m] * b1[q] + P[i + (int64_t)q * m] * b2[q];
    Y[(int64_t)(c0 + c) * ldy + s + i] = acc;
  }
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

void launch_leaf_dphiT(const double* Phi, const double* dPhi, int r, const Tree& t, const double* X,
                       int64_t ldx, double* VP, int k, cudaStream_t st) {
  dim3 grid((unsigned)t.nleaf, (unsigned)((k + 7) / 8));
  const size_t sm = (size_t)8 * t.max_leaf * sizeof(double);
  smem_limit((const void*)k_leaf_dphiT, sm);
  k_leaf_dphiT<<<grid, 256, sm, st>>>(Phi, dPhi, r, dtree(t), X, ldx, VP, k);
}

void launch_leaf_dnys_apply(const double* dKl, const double* Phi, const double* dPhi, const double* Sc,
                            const double* Sj, int r, const Tree& t, const double* X, int64_t ldx,
                            const double* VG, double* Y, int64_t ldy, int k, cudaStream_t st) {
  dim3 grid((unsigned)t.nleaf, (unsigned)((k + 7) / 8));
  const size_t sm = (size_t)8 * (t.max_leaf + 3 * r) * sizeof(double);
  smem_limit((const void*)k_leaf_dnys_apply, sm);
  k_leaf_dnys_apply<<<grid, 256, sm, st>>>(dKl, Phi, dPhi, Sc, Sj, r, dtree(t), X, ldx, VG, Y, ldy, k);
}

void launch_col_dots(const double* A, int64_t lda, const double* B, int64_t ldb, int64_t n, int k,
                     double* out, cudaStream_t st) {
  k_col_dots<<<k, 256, 0, st>>>(A, lda, B, ldb, n, out);
}

}  // namespace km
