// Covariance entries in float pairs (the mixed form) and the three first derivatives of an
// entry in one evaluation, shared by the assembly (km_assemble.cu) and the gradient (km_grad.cu).
#pragma once
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

// dkernel_value_ff for the three parameters at once, as float pairs (the same formulas; one
// float-pair exponential for the scale and range derivatives of the Matern kernel).
__device__ __forceinline__ void dkernel3_ff(const KParams& kp, double x1, double y1, double x2, double y2,
                                            ff (&out)[3]) {
  out[2] = (x1 == x2 && y1 == y2) ? ff(1.0) : ff(0.0);
  const ff dx(__dsub_rn(x1, x2)), dy(__dsub_rn(y1, y2));
  const ff r2 = ff(dx * dx) + dy * dy;
  const ff r = sqrt(r2);
  if (kp.kid == KM_KERNEL_RATQUAD) {
    const ff t = r / ff(kp.p1);
    const ff u = ff(1.0) + t * t;
    out[0] = ff(ff(2.0) * ff(kp.p0)) / ff(u * u);
    const ff num = ff(ff(4.0) * ff(ff(kp.p0) * ff(kp.p0))) * r2;
    const ff p13 = ff(ff(kp.p1) * ff(kp.p1)) * ff(kp.p1);
    out[1] = (num / p13) / ff(ff(u * u) * u);
    return;
  }
  out[0] = ff(1.0);
  out[1] = ff(0.0);
  if (!(r.hi > 0.f)) return;
  const ff x = r / ff(kp.p1);
  if (!(x.hi > 1.0e-8f)) return;
  const ff z = ff(kSqrt3) * x;
  const ff e = ff_exp_neg(z);
  out[0] = ff((ff(1.0) + z) * e);
  const ff num = ff(ff(3.0) * ff(kp.p0)) * ff(x * e);
  out[1] = ff(num * r) / ff(ff(kp.p1) * ff(kp.p1));
}

}  // namespace km
