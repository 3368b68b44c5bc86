// Kernel-entry evaluation: dense leaves, the Nystrom landmark columns Phi = K(X, P) and the
// landmark matrix S = K(P, P).  Replaces the comprehension in getindex/full
// (src/baseoverloads.jl:10-29) that KernelHODLR calls for every leaf (src/HODLR/src/
// constructor.jl:39) and nystrom_uvt calls for every block (src/factorizations.jl:86-94).
//
// Layouts (device):
//   points   : 2n doubles, (x, y) pairs (AoS, the SVector{2,Float64} layout)
//   leaves   : packed m_j x m_j column-major blocks at d_leaf_koff(j)
//   panels   : per-leaf m_j x r column-major blocks at leaf_start(j) * r
#include "km_kernels.h"

namespace km {

// ---------------------------------------------------------------------------------------------
// Float-pair evaluation for the mixed form.  The FP64 evaluation is bound by the FP64 pipe
// (sqrt, two divisions and exp per entry); here only the coordinate differences are formed in
// FP64 and everything else runs on the FP32 pipe in float pairs, to about 1e-14 relative
// (entries below 1e-37 round to 0).
//
// exp(-z), z >= 0: Cody-Waite reduction z = k ln2 + f with k = rint(z / ln2), |f| <= ln2/2, and
// the Taylor series of exp(-f) to degree 13 (remainder < 2e-16 for |f| <= 0.347), scaled by
// 2^-k.  The constants are the mathematical values ln 2 and 1/i!, rounded to float pairs.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ ff ff_exp_neg(ff z) {
  if (!(z.hi < 87.0f)) return ff(0.f, 0.f);
  // ln 2 as three floats (h + l + t); k*h and k*l are exact float pairs (FMA error terms), k*t
  // is far below the pair's precision
  constexpr double kLn2 = 0.69314718055994530942;
  constexpr float h = static_cast<float>(kLn2);
  constexpr float l = static_cast<float>(kLn2 - static_cast<double>(h));
  constexpr float t = static_cast<float>((kLn2 - static_cast<double>(h)) - static_cast<double>(l));
  const float k = rintf(z.hi * 1.44269504088896341f);
  const float kh = __fmul_rn(k, h), kl = __fmul_rn(k, l);
  const ff khp(kh, __fmaf_rn(k, h, -kh)), klp(kl, __fmaf_rn(k, l, -kl));
  const ff u = ((khp - z) + klp) + ff(__fmul_rn(k, t), 0.f);  // -(z - k ln2)
  constexpr double c[14] = {1.0, 1.0, 1.0 / 2, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720, 1.0 / 5040,
                            1.0 / 40320, 1.0 / 362880, 1.0 / 3628800, 1.0 / 39916800, 1.0 / 479001600,
                            1.0 / 6227020800.0};
  ff p(c[13]);
#pragma unroll
  for (int i = 12; i >= 0; --i) p = ff(c[i]) + p * u;
  const float sc = __int_as_float((127 - (int)k) << 23);  // 2^-k, k in [0, 126)
  return ff(p.hi * sc, p.lo * sc);
}

// kernel_value (km_internal.h) in float pairs, without the nugget; the same formulas and
// special cases.
__device__ __forceinline__ ff kernel_value_ffv(const KParams& kp, double x1, double y1, double x2, double y2) {
  const ff dx(__dsub_rn(x1, x2)), dy(__dsub_rn(y1, y2));
  const ff r = sqrt(ff(dx * dx) + dy * dy);
  ff out;
  if (kp.kid == KM_KERNEL_RATQUAD) {
    const ff t = r / ff(kp.p1);
    const ff u = ff(1.0) + t * t;
    out = ff(ff(kp.p0) * ff(kp.p0)) / ff(u * u);
  } else {
    out = ff(kp.p0);
    if (r.hi > 0.f) {
      const ff x = r / ff(kp.p1);
      if (x.hi > 1.0e-8f) {
        const ff z = ff(kSqrt3) * x;
        out = ff(ff(kp.p0) * (ff(1.0) + z)) * ff_exp_neg(z);
      }
    }
  }
  return out;
}

__device__ __forceinline__ double kernel_value_ff(const KParams& kp, double x1, double y1, double x2, double y2) {
  double v = to_double(kernel_value_ffv(kp, x1, y1, x2, y2));
  if (x1 == x2 && y1 == y2) v = __dadd_rn(v, kp.p2);
  return v;
}

// dkernel_value (km_internal.h) in float pairs.
__device__ __forceinline__ double dkernel_value_ff(const KParams& kp, int j, double x1, double y1, double x2,
                                                   double y2) {
  const bool same = (x1 == x2 && y1 == y2);
  if (j == 2) return same ? 1.0 : 0.0;
  const ff dx(__dsub_rn(x1, x2)), dy(__dsub_rn(y1, y2));
  const ff r2 = ff(dx * dx) + dy * dy;
  const ff r = sqrt(r2);
  if (kp.kid == KM_KERNEL_RATQUAD) {
    const ff t = r / ff(kp.p1);
    const ff u = ff(1.0) + t * t;
    if (j == 0) return to_double(ff(ff(2.0) * ff(kp.p0)) / ff(u * u));
    const ff num = ff(ff(4.0) * ff(ff(kp.p0) * ff(kp.p0))) * r2;
    const ff p13 = ff(ff(kp.p1) * ff(kp.p1)) * ff(kp.p1);
    return to_double((num / p13) / ff(ff(u * u) * u));
  }
  if (j == 0) {
    if (!(r.hi > 0.f)) return 1.0;
    const ff x = r / ff(kp.p1);
    if (!(x.hi > 1.0e-8f)) return 1.0;
    const ff z = ff(kSqrt3) * x;
    return to_double(ff((ff(1.0) + z)) * ff_exp_neg(z));
  }
  if (!(r.hi > 0.f)) return 0.0;
  const ff x = r / ff(kp.p1);
  if (!(x.hi > 1.0e-8f)) return 0.0;
  // -p0 * cor'(x) * r / p1^2 with cor'(x) = -3 x exp(-sqrt3 x)
  const ff e = ff_exp_neg(ff(kSqrt3) * x);
  const ff num = ff(ff(3.0) * ff(kp.p0)) * ff(x * e);
  return to_double(ff(num * r) / ff(ff(kp.p1) * ff(kp.p1)));
}

__device__ __forceinline__ double eval_entry(bool use_ff, const KParams& kp, int deriv, double x1, double y1,
                                             double x2, double y2) {
  if (deriv >= kD2Base)  // second derivatives: FP64 only
    return d2kernel_value(kp, (deriv - kD2Base) / 3, (deriv - kD2Base) % 3, x1, y1, x2, y2);
  if (use_ff)
    return deriv < 0 ? kernel_value_ff(kp, x1, y1, x2, y2) : dkernel_value_ff(kp, deriv, x1, y1, x2, y2);
  return deriv < 0 ? kernel_value(kp, x1, y1, x2, y2) : dkernel_value(kp, deriv, x1, y1, x2, y2);
}

// One 32x32 tile of one leaf per CTA; only lower-triangle tiles are evaluated and each is
// written twice (the kernel is symmetric bit for bit: |x-y| and x == y are symmetric).
// Kff (the kernel itself in float pairs, may be null): the entries of the evaluated tiles
// (every lower-triangle entry) also as float pairs, for the tensor-core leaf factorisation;
// the same kernel on the same points always gives the same pairs.
// grid = (ntile, ntile, nleaf), block = (32, 8).
__global__ void k_eval_leaves(const double* __restrict__ pts, DTree t, KParams kp, int deriv, bool use_ff,
                              double* __restrict__ K, ff* __restrict__ Kff) {
  const int ti = blockIdx.x, tj = blockIdx.y;
  if (ti < tj) return;
  const int64_t leaf = blockIdx.z;
  const int m = d_leaf_size(t, leaf);
  if (ti * 32 >= m) return;
  const int64_t s = d_leaf_start(t, leaf);
  double* A = K + d_leaf_koff(t, leaf);
  __shared__ double px[2][32], py[2][32];
  __shared__ double tile[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = ty * 32 + tx;
  if (tid < 64) {
    const int which = tid >> 5, q = tid & 31;
    const int idx = (which == 0 ? ti : tj) * 32 + q;
    if (idx < m) {
      px[which][q] = pts[2 * (s + idx)];
      py[which][q] = pts[2 * (s + idx) + 1];
    }
  }
  __syncthreads();
  const int i = ti * 32 + tx;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int jl = ty + 8 * q;
    const int j = tj * 32 + jl;
    if (i < m && j < m) {
      double v;
      if (Kff) {
        const double x1 = px[0][tx], y1 = py[0][tx], x2 = px[1][jl], y2 = py[1][jl];
        ff f = kernel_value_ffv(kp, x1, y1, x2, y2);
        v = to_double(f);
        if (x1 == x2 && y1 == y2) {  // the diagonal: the FP64 sum with the nugget, rounded to a pair
          v = __dadd_rn(v, kp.p2);
          f = ff(v);
        }
        Kff[d_leaf_koff(t, leaf) + (int64_t)j * m + i] = f;
      } else {
        v = eval_entry(use_ff, kp, deriv, px[0][tx], py[0][tx], px[1][jl], py[1][jl]);
      }
      A[(int64_t)j * m + i] = v;
      tile[tx][jl] = v;
    }
  }
  if (ti == tj) return;
  __syncthreads();
  // mirrored write: element (row = tj*32+tx, col = ti*32+ty+8q) = tile[ty+8q][tx]
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int il = ty + 8 * q;
    const int row = tj * 32 + tx, col = ti * 32 + il;
    if (row < m && col < m) A[(int64_t)col * m + row] = tile[il][tx];
  }
}

// Phi[i, c] = k(x_i, p_c) for every point i and landmark c, stored per leaf column-major.
// grid = (ceil(maxleaf*r / 256), nleaf), block = 256.
__global__ void k_eval_phi(const double* __restrict__ pts, const double* __restrict__ lnd, int r,
                           DTree t, KParams kp, int deriv, bool use_ff, double* __restrict__ Phi) {
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
  Phi[s * r + (int64_t)c * m + i] = eval_entry(use_ff, kp, deriv, x, y, sl[2 * c], sl[2 * c + 1]);
}

// Dense block out[i + j*ld] = k(a_i, b_j) (or its derivative) for small matrices such as S.
__global__ void k_eval_dense(const double* __restrict__ a, int na, const double* __restrict__ b,
                             int nb, KParams kp, int deriv, double* __restrict__ out, int ld) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= na * nb) return;
  const int i = e % na, j = e / na;
  const double v = eval_entry(false, kp, deriv, a[2 * i], a[2 * i + 1], b[2 * j], b[2 * j + 1]);
  out[i + (int64_t)j * ld] = v;
}

// Gathers the landmark points lnd[c] = pts[idx[c]].
__global__ void k_gather_points(const double* __restrict__ pts, const int64_t* __restrict__ idx,
                                int r, double* __restrict__ lnd) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < r) {
    lnd[2 * c] = pts[2 * idx[c]];
    lnd[2 * c + 1] = pts[2 * idx[c] + 1];
  }
}

void launch_eval_leaves(const double* pts, const Tree& t, KParams kp, int deriv, double* K,
                        cudaStream_t st, bool use_ff, ff* Kff) {
  const int nt = (int)((t.max_leaf + 31) / 32);
  dim3 grid(nt, nt, (unsigned)t.nleaf), block(32, 8);
  k_eval_leaves<<<grid, block, 0, st>>>(pts, dtree(t), kp, deriv, use_ff, K,
                                        (use_ff && deriv < 0) ? Kff : nullptr);
}

void launch_eval_phi(const double* pts, const double* lnd, int r, const Tree& t, KParams kp,
                     int deriv, double* Phi, cudaStream_t st, bool use_ff) {
  const int64_t per = t.max_leaf * r;
  dim3 grid((unsigned)((per + 255) / 256), (unsigned)t.nleaf);
  k_eval_phi<<<grid, 256, 2 * r * sizeof(double), st>>>(pts, lnd, r, dtree(t), kp, deriv, use_ff, Phi);
}

void launch_eval_dense(const double* a, int na, const double* b, int nb, KParams kp, int deriv,
                       double* out, int ld, cudaStream_t st) {
  const int tot = na * nb;
  k_eval_dense<<<(tot + 255) / 256, 256, 0, st>>>(a, na, b, nb, kp, deriv, out, ld);
}

void launch_gather_points(const double* pts, const int64_t* idx, int r, double* lnd,
                          cudaStream_t st) {
  k_gather_points<<<(r + 127) / 128, 128, 0, st>>>(pts, idx, r, lnd);
}

}  // namespace km
