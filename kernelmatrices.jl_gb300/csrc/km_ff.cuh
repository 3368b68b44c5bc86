// Float-float ("double-single") arithmetic for the mixed-precision form.
//
// GB300 issues FP32 FMAs 64x faster than FP64 ones (128 vs 2 per clock per SM).  A value is kept
// as an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2), which carries about 48
// significant bits.  The operations below are the classical error-free transformations
// (Knuth's TwoSum, Dekker's FastTwoSum, TwoProd via a fused multiply-add) combined as in the
// double-double algorithms of Dekker (1971) and Hida, Li and Bailey (2001), specialised to
// float pairs.  They need IEEE round-to-nearest float operations without reassociation
// (nvcc does not reassociate float arithmetic).
#pragma once
#include <cuda_runtime.h>
#ifndef __CUDA_ARCH__
#include <cstring>
#endif

namespace km {

// keep the standard overloads visible next to the float-pair ones declared below
using ::exp;
using ::fabs;
using ::fmax;
using ::fmin;
using ::log;
using ::sqrt;

// Exact float -> double conversion on the integer pipes, from the IEEE-754 binary32 and binary64
// layouts: the sign stays, a normal float's biased exponent E becomes E - 127 + 1023 and its 23
// significand bits move up by 29; a subnormal float M 2^-149 is normalised at its leading bit p
// (exponent p - 149, significand M shifted up by 52 - p without that bit); zeros keep their sign,
// infinities and NaNs keep the all-ones exponent and the payload.  Every float is a double, so
// the result equals the hardware conversion, which on GB300 runs on the FP64 pipe (2 lanes per
// clock per SM) and had bounded the kernels that write FP64 copies of float-pair values.
__host__ __device__ __forceinline__ unsigned long long f2d_bits(unsigned u) {
  const unsigned long long s = (unsigned long long)(u >> 31) << 63;
  const unsigned E = (u >> 23) & 0xffu, M = u & 0x7fffffu;
  if (E == 0xffu) return s | (0x7ffull << 52) | ((unsigned long long)M << 29);
  if (E != 0u) return s | ((unsigned long long)(E + 896u) << 52) | ((unsigned long long)M << 29);
  if (M == 0u) return s;
#ifdef __CUDA_ARCH__
  const int p = 31 - __clz((int)M);
#else
  const int p = 31 - __builtin_clz(M);
#endif
  return s | ((unsigned long long)(p + 874) << 52) | (((unsigned long long)M << (52 - p)) & 0xfffffffffffffull);
}

__host__ __device__ __forceinline__ double f2d_exact(float f) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)f2d_bits(__float_as_uint(f)));
#else
  unsigned u;
  std::memcpy(&u, &f, sizeof u);
  const unsigned long long b = f2d_bits(u);
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
#endif
}

struct __align__(8) ff {  // 8-byte aligned: one 64-bit load or store per value
  float hi, lo;
  __host__ __device__ constexpr ff() : hi(0.f), lo(0.f) {}
  __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
  // rounding a double to the nearest float pair (plain round-to-nearest casts, so that
  // constants such as ff(0.0) or ff(1.0) fold at compile time and cost no FP64 instruction)
  __host__ __device__ constexpr ff(double x) : hi(static_cast<float>(x)), lo(static_cast<float>(x - static_cast<double>(static_cast<float>(x)))) {}
  // hi + lo rounded to a double: the exact conversions of both parts and one FP64 add, the same
  // value as (double)hi + (double)lo
  __device__ explicit operator double() const { return __dadd_rn(f2d_exact(hi), f2d_exact(lo)); }
};

__device__ __forceinline__ void ff_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void ff_fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}

__device__ __forceinline__ ff operator+(ff a, ff b) {
  float s, e;
  ff_two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  ff r;
  ff_fast_two_sum(s, e, r.hi, r.lo);
  return r;
}

__device__ __forceinline__ ff operator-(ff a) { return ff(-a.hi, -a.lo); }
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }

// A product is returned unnormalised (p + e with e the exact rounding error of a.hi*b.hi plus
// the cross terms) and normalised only when it is used as a value.  acc + a*b and acc - a*b
// then add (p, e) to acc directly, which saves the intermediate FastTwoSum: 15 FP32
// instructions per multiply-add instead of 18.
struct ffprod {
  float p, e;
  __device__ __forceinline__ operator ff() const {
    ff r;
    ff_fast_two_sum(p, e, r.hi, r.lo);
    return r;
  }
};

__device__ __forceinline__ ffprod operator*(ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return ffprod{p, e};
}

__device__ __forceinline__ ff operator+(ff a, ffprod b) {
  float s, t;
  ff_two_sum(a.hi, b.p, s, t);
  t = __fadd_rn(t, __fadd_rn(a.lo, b.e));
  ff r;
  ff_fast_two_sum(s, t, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ ff operator+(ffprod b, ff a) { return a + b; }
__device__ __forceinline__ ff operator-(ff a, ffprod b) { return a + ffprod{-b.p, -b.e}; }
__device__ __forceinline__ ff operator-(ffprod b) { return ff(ffprod{-b.p, -b.e}); }
__device__ __forceinline__ ff operator+(ffprod a, ffprod b) { return ff(a) + b; }
__device__ __forceinline__ ff operator-(ffprod a, ffprod b) { return ff(a) - b; }
__device__ __forceinline__ ff operator-(ffprod a, ff b) { return ff(a) - b; }
__device__ __forceinline__ ffprod operator*(ffprod a, ff b) { return ff(a) * b; }
__device__ __forceinline__ ffprod operator*(ff a, ffprod b) { return a * ff(b); }
__device__ __forceinline__ ffprod operator*(ffprod a, ffprod b) { return ff(a) * ff(b); }

__device__ __forceinline__ ff operator/(ff a, ff b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const ff r = a - b * ff(q1, 0.f);
  const float q2 = __fdiv_rn(r.hi, b.hi);
  ff out;
  ff_fast_two_sum(q1, q2, out.hi, out.lo);
  return out;
}

__device__ __forceinline__ ff& operator+=(ff& a, ff b) { return a = a + b; }
__device__ __forceinline__ ff& operator-=(ff& a, ff b) { return a = a - b; }
__device__ __forceinline__ ff& operator+=(ff& a, ffprod b) { return a = a + b; }
__device__ __forceinline__ ff& operator-=(ff& a, ffprod b) { return a = a - b; }
__device__ __forceinline__ ff& operator*=(ff& a, ff b) { return a = ff(a * b); }
__device__ __forceinline__ ff& operator/=(ff& a, ff b) { return a = a / b; }

// Dot-product accumulator in the manner of Dot2 (Ogita, Rump and Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26, 2005): the high parts are summed with TwoSum and every
// rounding error (TwoSum's and the product's) is summed in a plain float, renormalised once when
// the value is read.  The loop-carried dependency is a single float add per term (the
// renormalising accumulate carries nine), and a multiply-add costs 12 FP32 instructions; the
// result is as accurate as if the sum were formed in twice the float precision.
struct ffacc {
  float s, c;
  __device__ __forceinline__ constexpr ffacc() : s(0.f), c(0.f) {}
  __device__ __forceinline__ constexpr ffacc(ff a) : s(a.hi), c(a.lo) {}
  __device__ __forceinline__ void add(float x, float ex) {
    const float t = __fadd_rn(s, x);
    const float bb = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(x, bb));
    s = t;
    c = __fadd_rn(c, __fadd_rn(e, ex));
  }
  __device__ __forceinline__ ff value() const {
    ff r;
    ff_two_sum(s, c, r.hi, r.lo);
    return r;
  }
};
__device__ __forceinline__ ffacc& operator+=(ffacc& a, ffprod b) { a.add(b.p, b.e); return a; }
__device__ __forceinline__ ffacc& operator-=(ffacc& a, ffprod b) { a.add(-b.p, -b.e); return a; }
__device__ __forceinline__ ffacc& operator+=(ffacc& a, ff b) { a.add(b.hi, b.lo); return a; }
__device__ __forceinline__ ffacc& operator-=(ffacc& a, ff b) { a.add(-b.hi, -b.lo); return a; }

// acc_t<T>: the accumulator of a sum of T terms (T itself for double); accv reads its value.
template <typename T> struct AccOf { using type = T; };
template <> struct AccOf<ff> { using type = ffacc; };
template <typename T> using acc_t = typename AccOf<T>::type;
__device__ __forceinline__ double accv(double a) { return a; }
__device__ __forceinline__ ff accv(const ffacc& a) { return a.value(); }

// Comparisons with a double constant b, in float arithmetic.  Exact when b is a float pair
// (b == ff(b)), which holds for the constants the kernels compare with (0, 1).  For a normalised
// pair the order is decided by hi, and by lo when the hi parts are equal.
__device__ __forceinline__ bool operator>(ff a, double b) {
  const ff c(b);
  return a.hi > c.hi || (a.hi == c.hi && a.lo > c.lo);
}
__device__ __forceinline__ bool operator>=(ff a, double b) {
  const ff c(b);
  return a.hi > c.hi || (a.hi == c.hi && a.lo >= c.lo);
}
__device__ __forceinline__ bool operator==(ff a, double b) {
  const ff c(b);
  return a.hi == c.hi && a.lo == c.lo;
}
__device__ __forceinline__ bool operator!=(ff a, double b) { return !(a == b); }

// sqrt(a): the fast approximate float square root (s = a.hi rsqrt(a.hi)) corrected by one
// Newton step in float pairs, s + (a - s^2) / (2 s); relative error about 1e-13.
__device__ __forceinline__ ff sqrt(ff a) {
  if (!(a.hi > 0.f)) return ff(0.f, 0.f);
  const float rs = rsqrtf(a.hi);
  const float s = __fmul_rn(a.hi, rs);
  const ff r = a - ff(s, 0.f) * ff(s, 0.f);
  const float c = __fmul_rn(r.hi, __fmul_rn(0.5f, rs));  // (a - s^2) / (2 s), 1/s ~ rsqrt(a)
  ff out;
  ff_fast_two_sum(s, c, out.hi, out.lo);
  return out;
}

// 1 / b: the fast approximate float reciprocal refined by one Newton step in float pairs,
// y + y (1 - b y) (relative error about 1e-13).  A much shorter dependency chain than a / b,
// for pivots on a critical path.
__device__ __forceinline__ ff ff_recip(ff b) {
  const ff y(__fdividef(1.0f, b.hi), 0.f);
  const ff e = ff(1.0f, 0.f) - b * y;
  return y + y * e;
}
__device__ __forceinline__ double ff_recip(double b) { return 1.0 / b; }

__device__ __forceinline__ ff fabs(ff a) { return a.hi < 0.f ? -a : a; }

__device__ __forceinline__ ff shfl_xor(ff v, int o) {
  return ff(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
}
__device__ __forceinline__ ff shfl_idx(ff v, int src) {
  return ff(__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src));
}
__device__ __forceinline__ double shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double shfl_idx(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }

template <typename T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = v + shfl_xor(v, o);
  return v;
}

// conversions used at buffer boundaries
template <typename T> __device__ __forceinline__ T from_double(double x);
template <> __device__ __forceinline__ double from_double<double>(double x) { return x; }
template <> __device__ __forceinline__ ff from_double<ff>(double x) { return ff(x); }
__device__ __forceinline__ double to_double(double x) { return x; }
__device__ __forceinline__ double to_double(ff x) { return (double)x; }

}  // namespace km
