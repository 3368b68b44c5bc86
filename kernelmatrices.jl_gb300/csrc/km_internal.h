// Internal definitions shared by the CUDA translation units of libkmhodlr.
//
// Tree layout (all 0-based):
//   * leaves j = 0 .. nleaf-1, nleaf = 2^L.  The first `rem` leaves hold m0+1 points, the rest m0
//     (src/HODLR/src/indices.jl:5-24 gives the remainder to the first leaves), so
//     start(j) = j*m0 + min(j, rem) and size(j) = m0 + (j < rem).
//   * level l = 1..L holds 2^(L-l) nodes; node k of level l has children 2k (first, earlier
//     rows, the reference's columns c:d) and 2k+1 (second, the reference's rows a:b) of level l-1,
//     level 0 being the leaves (src/HODLR/src/indices.jl:40-51).
//   * "slots" number leaves and nodes together: slot(leaf j) = j, slot(level l, node k) =
//     nleaf + node_off[l] + k with node_off[1] = 0.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/kmhodlr.h"

namespace km {

constexpr int kMaxNysRank = 80;     // Nystrom rank bound of the nested factorisation kernels
constexpr int kMaxLevels = 40;

struct Tree {
  int64_t n = 0;
  int L = 0;            // number of levels
  int64_t m0 = 0;       // base leaf size
  int64_t rem = 0;      // leaves with m0+1 points
  int64_t nleaf = 0;
  int64_t nnode = 0;    // 2^L - 1
  int64_t max_leaf = 0;
  std::vector<int64_t> node_off;  // size L+2, node_off[l] for l = 1..L+1

  int64_t leaf_start(int64_t j) const { return j * m0 + (j < rem ? j : rem); }
  int64_t leaf_size(int64_t j) const { return m0 + (j < rem ? 1 : 0); }
  int64_t nodes_at(int l) const { return int64_t(1) << (L - l); }
  int64_t slot(int l, int64_t k) const { return l == 0 ? k : nleaf + node_off[l] + k; }
  // first row and row count of node k at level l (level 0 = leaf)
  int64_t node_start(int l, int64_t k) const { return leaf_start(k << l); }
  int64_t node_size(int l, int64_t k) const {
    int64_t a = leaf_start(k << l);
    int64_t b = (((k + 1) << l) >= nleaf) ? n : leaf_start((k + 1) << l);
    return b - a;
  }
};

// Builds the tree from n and a level policy; returns false (with msg) on bad input.
bool build_tree(int64_t n, int level_kind, int64_t level, Tree* t, std::string* msg);

// Kernel parameters passed by value to device code.
struct KParams {
  int kid;          // km_kernel_id
  double p0, p1, p2;
  float p0h, p0l, p1h, p1l;  // p0 and p1 rounded to float pairs once (the float-pair evaluations)
  float ip1h, ip1l;          // 1 / p1 (FP64 division) rounded to a float pair
};

// KParams with the float-pair copies of p0, p1 and 1 / p1: hi = fl32(p), lo = fl32(p - hi), the
// rounding of the float-pair type's constructor
inline KParams make_kparams(int kid, double p0, double p1, double p2) {
  KParams k{kid, p0, p1, p2, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  k.p0h = static_cast<float>(p0);
  k.p0l = static_cast<float>(p0 - static_cast<double>(k.p0h));
  k.p1h = static_cast<float>(p1);
  k.p1l = static_cast<float>(p1 - static_cast<double>(k.p1h));
  const double ip1 = 1.0 / p1;
  k.ip1h = static_cast<float>(ip1);
  k.ip1l = static_cast<float>(ip1 - static_cast<double>(k.ip1h));
  return k;
}

// Device-side tree description passed by value.
struct DTree {
  int64_t n, m0, rem, nleaf;
  int L;
};

inline DTree dtree(const Tree& t) { return DTree{t.n, t.m0, t.rem, t.nleaf, t.L}; }

}  // namespace km

// ----------------------------------------------------------------------------------------------
// Device helpers
// ----------------------------------------------------------------------------------------------
#ifdef __CUDACC__
namespace km {

__host__ __device__ inline int64_t d_leaf_start(const DTree& t, int64_t j) {
  return j * t.m0 + (j < t.rem ? j : t.rem);
}
__host__ __device__ inline int d_leaf_size(const DTree& t, int64_t j) {
  return (int)(t.m0 + (j < t.rem ? 1 : 0));
}
// offset of leaf j's m x m block in the packed leaf storage (sum of previous sizes squared)
__host__ __device__ inline int64_t d_leaf_koff(const DTree& t, int64_t j) {
  const int64_t big = (j < t.rem ? j : t.rem);
  const int64_t small = j - big;
  return big * (t.m0 + 1) * (t.m0 + 1) + small * t.m0 * t.m0;
}

constexpr double kSqrt3 = 1.7320508075688772;

// Covariance value.  Written with explicit round-to-nearest operations (no fused multiply-add)
// so that it rounds exactly like the NumPy restatement of the reference:
//   RATQUAD : p0^2 / (1 + (r/p1)^2)^2          (README.md:42-48)
//   MATERN32: p0 * (1 + z) exp(-z), z = sqrt3 r/p1 when r > 0 and r/p1 > 1e-8, else p0
//             (mtn_kernfun / mtn_cor, src/covariancefunctions.jl:209-212, 258-266)
// plus p2 when the two points are equal coordinate by coordinate (x == y).
__device__ __forceinline__ double kernel_value(const KParams& kp, double x1, double y1, double x2,
                                               double y2) {
  const double dx = __dsub_rn(x1, x2), dy = __dsub_rn(y1, y2);
  const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
  double out;
  if (kp.kid == KM_KERNEL_RATQUAD) {
    const double t = __ddiv_rn(r, kp.p1);
    const double u = __dadd_rn(1.0, __dmul_rn(t, t));
    out = __ddiv_rn(__dmul_rn(kp.p0, kp.p0), __dmul_rn(u, u));
  } else {
    out = kp.p0;
    if (r > 0.0) {
      const double x = __ddiv_rn(r, kp.p1);
      if (fabs(x) > 1.0e-8) {
        const double z = __dmul_rn(kSqrt3, x);
        out = __dmul_rn(kp.p0, __dmul_rn(__dadd_rn(1.0, z), exp(-z)));
      }
    }
  }
  if (x1 == x2 && y1 == y2) out = __dadd_rn(out, kp.p2);
  return out;
}

// Derivative of kernel_value in parameter `j` (0 scale, 1 range, 2 nugget):
//   MATERN32: mtn_kernfun_d1 / _d2 (src/covariancefunctions.jl:268-286) at nu = 3/2;
//   RATQUAD : 2 p0/u^2 and 4 p0^2 r^2/(p1^3 u^3);
//   nugget  : [x == y].
__device__ __forceinline__ double dkernel_value(const KParams& kp, int j, double x1, double y1,
                                                double x2, double y2) {
  const bool same = (x1 == x2 && y1 == y2);
  if (j == 2) return same ? 1.0 : 0.0;
  const double dx = __dsub_rn(x1, x2), dy = __dsub_rn(y1, y2);
  const double r2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  const double r = __dsqrt_rn(r2);
  if (kp.kid == KM_KERNEL_RATQUAD) {
    const double t = __ddiv_rn(r, kp.p1);
    const double u = __dadd_rn(1.0, __dmul_rn(t, t));
    if (j == 0) return __ddiv_rn(__dmul_rn(2.0, kp.p0), __dmul_rn(u, u));
    const double num = __dmul_rn(__dmul_rn(4.0, __dmul_rn(kp.p0, kp.p0)), __dmul_rn(r, r));
    const double p13 = __dmul_rn(__dmul_rn(kp.p1, kp.p1), kp.p1);
    return __ddiv_rn(__ddiv_rn(num, p13), __dmul_rn(__dmul_rn(u, u), u));
  }
  if (j == 0) {
    if (!(r > 0.0)) return 1.0;
    const double x = __ddiv_rn(r, kp.p1);
    if (!(fabs(x) > 1.0e-8)) return 1.0;
    const double z = __dmul_rn(kSqrt3, x);
    return __dmul_rn(__dadd_rn(1.0, z), exp(-z));
  }
  if (!(r > 0.0)) return 0.0;
  const double x = __ddiv_rn(r, kp.p1);
  if (!(fabs(x) > 1.0e-8)) return 0.0;
  // -p0 * cor'(x) * r / p1^2 with cor'(x) = -3 x exp(-sqrt3 x)
  const double dc = __dmul_rn(__dmul_rn(-3.0, x), exp(-__dmul_rn(kSqrt3, x)));
  return __ddiv_rn(__dmul_rn(__dmul_rn(-kp.p0, dc), r), __dmul_rn(kp.p1, kp.p1));
}

// Second derivative of kernel_value in parameters j and k (0 scale, 1 range, 2 nugget), the
// closed forms of the second-derivative functions the reference's stoch_hessian takes from its
// caller (d2funs, src/HODLR/src/stochastichessian.jl:117-121):
//   MATERN32 (z = sqrt3 r / p1): d00 = 0, d01 = z^2 e^-z / p1, d11 = p0 z^2 (z - 3) e^-z / p1^2,
//            0 where r / p1 <= 1e-8 as for the first derivative;
//   RATQUAD  (u = 1 + t^2, t = r / p1): d00 = 2 / u^2, d01 = 8 p0 r^2 / (p1^3 u^3),
//            d11 = 12 p0^2 r^2 (t^2 - 1) / (p1^4 u^4);
//   any pair with the nugget: 0.
// Evaluation kernels select it with deriv = kD2Base + 3 j + k.
constexpr int kD2Base = 10;

__device__ __forceinline__ double d2kernel_value(const KParams& kp, int j, int k, double x1, double y1,
                                                 double x2, double y2) {
  if (j > k) {
    const int s = j;
    j = k;
    k = s;
  }
  if (k == 2) return 0.0;
  const double dx = x1 - x2, dy = y1 - y2;
  const double r2 = dx * dx + dy * dy;
  const double r = sqrt(r2);
  if (kp.kid == KM_KERNEL_RATQUAD) {
    const double t = r / kp.p1;
    const double u = 1.0 + t * t;
    if (j == 0 && k == 0) return 2.0 / (u * u);
    const double p13 = kp.p1 * kp.p1 * kp.p1;
    if (j == 0) return 8.0 * kp.p0 * r2 / p13 / (u * u * u);
    return 12.0 * kp.p0 * kp.p0 * r2 * (t * t - 1.0) / (p13 * kp.p1) / (u * u * u * u);
  }
  if (j == 0 && k == 0) return 0.0;
  if (!(r > 0.0)) return 0.0;
  const double x = r / kp.p1;
  if (!(fabs(x) > 1.0e-8)) return 0.0;
  const double z = kSqrt3 * x;
  const double e = exp(-z);
  if (j == 0) return z * z * e / kp.p1;
  return kp.p0 * z * z * (z - 3.0) * e / (kp.p1 * kp.p1);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace km
#endif  // __CUDACC__
