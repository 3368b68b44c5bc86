// Covariance entries in float pairs (the mixed form) and the three first derivatives of an
// entry in one evaluation, shared by the assembly (km_assemble.cu) and the gradient (km_grad.cu).
#pragma once
#include "km_kernels.h"

namespace km {

// ---------------------------------------------------------------------------------------------
// Float-pair evaluation for the mixed form.  The FP64 evaluation is bound by the FP64 pipe
// (sqrt, two divisions and exp per entry); here everything runs on the FP32 pipe in float pairs,
// to about 1e-14 relative (entries below 1e-37 round to 0).
//
// exp(-z), z >= 0: Cody-Waite reduction z = k ln2 + f with k = rint(z / ln2), |f| <= ln2/2, and
// the Taylor series of exp(-f) to degree 13 (remainder < 2e-16 for |f| <= 0.347), scaled by
// 2^-k.  The constants are the mathematical values ln 2 and 1/i!, rounded to float pairs.  The
// terms of degree 9 to 13 are below 2^-32 of the sum (0.347^9 / 9! = 2e-10), so their Horner
// steps run in plain floats on the high part of -f (errors below 2^-55 of the sum); the terms of
// degree 0 to 8 in float pairs.
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
  float q = static_cast<float>(c[13]);
#pragma unroll
  for (int i = 12; i >= 9; --i) q = __fmaf_rn(q, u.hi, static_cast<float>(c[i]));
  ff p = ff(c[8]) + ff(q, 0.f) * u;
#pragma unroll
  for (int i = 7; i >= 0; --i) p = ff(c[i]) + p * u;
  const float sc = __int_as_float((127 - (int)k) << 23);  // 2^-k, k in [0, 126)
  return ff(p.hi * sc, p.lo * sc);
}

// ---------------------------------------------------------------------------------------------
// Coordinates as exact float triples.  A double x is split into h = fl32(x), m = fl32(x - h),
// l = x - h - m (at most 7 significant bits, exact in a float), so x = h + m + l exactly; the
// points are split once per assembly (k_split_points) and the float-pair evaluations form the
// coordinate differences from the triples on the FP32 pipe, with no FP64 instruction: the FP64
// pipe (2 operations per clock per SM) had bounded the float-pair evaluation kernels on the
// conversions of the FP64 differences.  Two triples are equal component by component exactly
// when the doubles are equal (x == y, the nugget's test).
// ---------------------------------------------------------------------------------------------
// p0 and p1 as float pairs (rounded on the host once, KParams)
__device__ __forceinline__ ff kp_p0(const KParams& kp) { return ff(kp.p0h, kp.p0l); }
__device__ __forceinline__ ff kp_p1(const KParams& kp) { return ff(kp.p1h, kp.p1l); }
// 1 / p1 as a float pair: r / p1 is formed as r * (1 / p1), one float-pair product in place of a
// float-pair division (the same accuracy, about 2^-47 relative)
__device__ __forceinline__ ff kp_ip1(const KParams& kp) { return ff(kp.ip1h, kp.ip1l); }

struct f3 {
  float h, m, l;
};

__device__ __forceinline__ f3 split3(double x) {
  const float h = __double2float_rn(x);
  const double r1 = x - (double)h;  // exact
  const float m = __double2float_rn(r1);
  return f3{h, m, __double2float_rn(r1 - (double)m)};  // exact
}

__device__ __forceinline__ bool eq3(const f3& a, const f3& b) { return a.h == b.h && a.m == b.m && a.l == b.l; }

// the float pair nearest (to about 2^-48 relative, or far below the pair's precision in absolute
// terms) to a - b: the high and middle differences exactly by TwoSum, the low ones rounded
__device__ __forceinline__ ff ff_sub3(const f3& a, const f3& b) {
  float s, e, t, f;
  ff_two_sum(a.h, -b.h, s, e);
  ff_two_sum(a.m, -b.m, t, f);
  ff r = ff(s, e) + ff(t, f);
  return r + ff(__fsub_rn(a.l, b.l), 0.f);
}

// kernel_value (km_internal.h) in float pairs, without the nugget; the same formulas and
// special cases, on split coordinates, with r / p1 formed as r * (1 / p1).
__device__ __forceinline__ ff kernel_value_ffp(const KParams& kp, const f3& x1, const f3& y1, const f3& x2,
                                               const f3& y2) {
  const ff dx = ff_sub3(x1, x2), dy = ff_sub3(y1, y2);
  const ff r = sqrt(ff(dx * dx) + dy * dy);
  ff out;
  if (kp.kid == KM_KERNEL_RATQUAD) {
    const ff t = r * kp_ip1(kp);
    const ff u = ff(1.0) + t * t;
    out = ff(kp_p0(kp) * kp_p0(kp)) / ff(u * u);
  } else {
    out = kp_p0(kp);
    if (r.hi > 0.f) {
      const ff x = r * kp_ip1(kp);
      if (x.hi > 1.0e-8f) {
        const ff z = ff(kSqrt3) * x;
        out = ff(kp_p0(kp) * (ff(1.0) + z)) * ff_exp_neg(z);
      }
    }
  }
  return out;
}

__device__ __forceinline__ ff kernel_value_ffv(const KParams& kp, double x1, double y1, double x2, double y2) {
  return kernel_value_ffp(kp, split3(x1), split3(y1), split3(x2), split3(y2));
}

__device__ __forceinline__ double kernel_value_ff(const KParams& kp, double x1, double y1, double x2, double y2) {
  double v = to_double(kernel_value_ffv(kp, x1, y1, x2, y2));
  if (x1 == x2 && y1 == y2) v = __dadd_rn(v, kp.p2);
  return v;
}

// dkernel_value (km_internal.h) for the three parameters at once in float pairs, on split
// coordinates: one distance and, for the Matern kernel, one exponential shared by the scale and
// range derivatives; r / p1 formed as r * (1 / p1).
__device__ __forceinline__ void dkernel3_ffp(const KParams& kp, const f3& x1, const f3& y1, const f3& x2,
                                             const f3& y2, ff (&out)[3]) {
  out[2] = (eq3(x1, x2) && eq3(y1, y2)) ? ff(1.0) : ff(0.0);
  const ff dx = ff_sub3(x1, x2), dy = ff_sub3(y1, y2);
  const ff r2 = ff(dx * dx) + dy * dy;
  const ff r = sqrt(r2);
  if (kp.kid == KM_KERNEL_RATQUAD) {
    const ff t = r * kp_ip1(kp);
    const ff u = ff(1.0) + t * t;
    out[0] = ff(ff(2.0) * kp_p0(kp)) / ff(u * u);
    const ff num = ff(ff(4.0) * ff(kp_p0(kp) * kp_p0(kp))) * r2;
    const ff p13 = ff(kp_p1(kp) * kp_p1(kp)) * kp_p1(kp);
    out[1] = (num / p13) / ff(ff(u * u) * u);
    return;
  }
  out[0] = ff(1.0);
  out[1] = ff(0.0);
  if (!(r.hi > 0.f)) return;
  const ff x = r * kp_ip1(kp);
  if (!(x.hi > 1.0e-8f)) return;
  // -p0 * cor'(x) * r / p1^2 with cor'(x) = -3 x exp(-sqrt3 x)
  const ff z = ff(kSqrt3) * x;
  const ff e = ff_exp_neg(z);
  out[0] = ff((ff(1.0) + z) * e);
  const ff num = ff(ff(3.0) * kp_p0(kp)) * ff(x * e);
  out[1] = ff(num * r) / ff(kp_p1(kp) * kp_p1(kp));
}

__device__ __forceinline__ void dkernel3_ff(const KParams& kp, double x1, double y1, double x2, double y2,
                                            ff (&out)[3]) {
  dkernel3_ffp(kp, split3(x1), split3(y1), split3(x2), split3(y2), out);
}

// dkernel_value (km_internal.h) in float pairs.
__device__ __forceinline__ double dkernel_value_ff(const KParams& kp, int j, double x1, double y1, double x2,
                                                   double y2) {
  ff v[3];
  dkernel3_ff(kp, x1, y1, x2, y2, v);
  return to_double(v[j]);
}

// split coordinates of point i from the array of 8 floats a point (xh, xm, xl, yh, ym, yl, 0, 0)
__device__ __forceinline__ void load_p3(const float* __restrict__ P3, int64_t i, f3& x, f3& y) {
  const float4 a = *reinterpret_cast<const float4*>(P3 + 8 * i);
  const float4 b = *reinterpret_cast<const float4*>(P3 + 8 * i + 4);
  x = f3{a.x, a.y, a.z};
  y = f3{a.w, b.x, b.y};
}

__device__ __forceinline__ double eval_entry(bool use_ff, const KParams& kp, int deriv, double x1, double y1,
                                             double x2, double y2) {
  if (deriv >= kD2Base)  // second derivatives: FP64 only
    return d2kernel_value(kp, (deriv - kD2Base) / 3, (deriv - kD2Base) % 3, x1, y1, x2, y2);
  if (use_ff)
    return deriv < 0 ? kernel_value_ff(kp, x1, y1, x2, y2) : dkernel_value_ff(kp, deriv, x1, y1, x2, y2);
  return deriv < 0 ? kernel_value(kp, x1, y1, x2, y2) : dkernel_value(kp, deriv, x1, y1, x2, y2);
}

// dkernel_value (km_internal.h) for the three parameters at once: one distance and, for the
// Matern kernel, one exponential shared by the scale and range derivatives.  out[j] equals
// dkernel_value(kp, j, ...) bit for bit (the same operations in the same order).
__device__ __forceinline__ void dkernel3(const KParams& kp, double x1, double y1, double x2, double y2,
                                         double (&out)[3]) {
  out[2] = (x1 == x2 && y1 == y2) ? 1.0 : 0.0;
  const double dx = __dsub_rn(x1, x2), dy = __dsub_rn(y1, y2);
  const double r2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  const double r = __dsqrt_rn(r2);
  if (kp.kid == KM_KERNEL_RATQUAD) {
    const double t = __ddiv_rn(r, kp.p1);
    const double u = __dadd_rn(1.0, __dmul_rn(t, t));
    out[0] = __ddiv_rn(__dmul_rn(2.0, kp.p0), __dmul_rn(u, u));
    const double num = __dmul_rn(__dmul_rn(4.0, __dmul_rn(kp.p0, kp.p0)), __dmul_rn(r, r));
    const double p13 = __dmul_rn(__dmul_rn(kp.p1, kp.p1), kp.p1);
    out[1] = __ddiv_rn(__ddiv_rn(num, p13), __dmul_rn(__dmul_rn(u, u), u));
    return;
  }
  out[0] = 1.0;
  out[1] = 0.0;
  if (!(r > 0.0)) return;
  const double x = __ddiv_rn(r, kp.p1);
  if (!(fabs(x) > 1.0e-8)) return;
  const double z = __dmul_rn(kSqrt3, x);
  const double e = exp(-z);
  out[0] = __dmul_rn(__dadd_rn(1.0, z), e);
  const double dc = __dmul_rn(__dmul_rn(-3.0, x), e);
  out[1] = __ddiv_rn(__dmul_rn(__dmul_rn(-kp.p0, dc), r), __dmul_rn(kp.p1, kp.p1));
}

}  // namespace km
