// Blackwell (sm_103a) tensor-core and bulk-copy primitives, as inline PTX:
//   * mbarriers (init, expect-tx arrive, bounded parity wait),
//   * one-dimensional bulk copies global -> shared memory completing on an mbarrier (TMA engine),
//   * tcgen05: tensor-memory allocation, bf16 x bf16 -> fp32 MMA with operands in shared memory,
//     commit to an mbarrier, loads of the accumulator from tensor memory.
//
// Operand layout in shared memory: the canonical K-major layout without swizzling.  A "core
// matrix" is 8 rows x 16 bytes (8 bf16 along K) stored as 128 contiguous bytes (row r at byte
// 16 r).  The matrix descriptor gives the byte distance between core matrices adjacent along K
// (leading dimension offset) and along M / N (stride dimension offset).
//
// Split products.  A float-pair (or double) value x of a row whose largest magnitude is below
// 2^e is written as x = 2^e sum_{i<kSlices} t_i 2^{-7(i+1)} with integer slices t_0 in
// [-128, 128] and t_i in [-65, 65] (each slice is the rounded-to-nearest integer part of the
// remainder times 2^7).  Every slice is exactly a bf16 value.  The product of two rows is then
// 2^{e_a + e_b} sum_d 2^{-7(d+2)} s_d with s_d = sum_{i+j=d} sum_k t_i(a_k) t_j(b_k): each s_d
// is a sum of integer products below 2^23.3 in magnitude for K <= 256 (< 2^24), so the tensor
// core's fp32 accumulation forms it exactly.  Dropping the diagonals d >= kSlices costs
// about 2^{-7 kSlices} of the row scales, below the float-pair rounding for kSlices = 7.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "km_ff.cuh"

namespace km {
namespace tc {

constexpr int kSlices = 7;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- mbarriers -------------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the phase with the given parity to complete, giving up after `limit` polls (each
// poll may suspend the thread for a hardware-chosen time); returns false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit) {
  for (long long it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// ---- bulk copies (global -> shared, completing on an mbarrier) -------------------------------
// dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// generic-proxy writes to shared memory made visible to the async proxy (tensor core reads)
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- tensor memory ----------------------------------------------------------------------------
// Allocation by one full warp; the address is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor: start address, leading (K-direction) and stride (M/N
// direction) byte offsets between core matrices, descriptor version 1, no swizzling.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: fp32 accumulator, bf16 A and B, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D(tmem) (+)= A(smem) * B(smem)^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}
// Arrives on the mbarrier once every MMA issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// Eight consecutive 32-bit accumulator columns of this thread's lane (warp w reads lanes
// 32 (w % 4) .. 32 (w % 4) + 31).
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---- slices -----------------------------------------------------------------------------------
// Exponent e with max|x| < 2^e over a row (0 for a zero row).
__device__ __forceinline__ int row_exponent(float amax) {
  if (!(amax > 0.f)) return 0;
  int e;
  frexpf(amax, &e);  // amax = f 2^e, f in [0.5, 1)
  return e;
}

// 2^k as a float for -126 <= k <= 127
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((k + 127) << 23); }

// x * 2^k for a float pair, exact while no part leaves the normal range (|k| <= 250)
__device__ __forceinline__ ff ff_ldexp(ff x, int k) {
  const int k1 = k / 2, k2 = k - k1;
  const float s1 = pow2f(k1), s2 = pow2f(k2);
  return ff(x.hi * s1 * s2, x.lo * s1 * s2);
}

// The kSlices integer slices of x (|x| < 2^e), as floats (exact bf16 values).
__device__ __forceinline__ void split_slices(ff x, int e, float (&t)[kSlices]) {
  const float s = pow2f(7 - e);
  float h = x.hi * s, l = x.lo * s;  // exact scaling: |h + l| < 2^7
#pragma unroll
  for (int i = 0; i < kSlices; ++i) {
    const float ti = rintf(h);
    t[i] = ti;
    float a, b;
    ff_two_sum(h - ti, l, a, b);  // h - ti is exact
    h = a * 128.f;
    l = b * 128.f;
  }
}

// sum_d 2^{-7(d+2)} s_d (s_d exact integers < 2^24) as a float pair, smallest terms first
__device__ __forceinline__ ff combine_diagonals(const float (&s)[kSlices]) {
  ff acc(s[kSlices - 1] * pow2f(-7 * (kSlices + 1)), 0.f);
#pragma unroll
  for (int d = kSlices - 2; d >= 0; --d) {
    float hi, e;
    ff_two_sum(acc.hi, s[d] * pow2f(-7 * (d + 2)), hi, e);
    e += acc.lo;
    ff_fast_two_sum(hi, e, acc.hi, acc.lo);
  }
  return acc;
}

// bf16 bits of an exactly representable float (integers |v| <= 256 here)
__device__ __forceinline__ uint32_t bf16_pack2(float lo, float hi) {
  return (__float_as_uint(lo) >> 16) | (__float_as_uint(hi) & 0xFFFF0000u);
}

}  // namespace tc
}  // namespace km
