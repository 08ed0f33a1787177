// tc_common.cuh -- device helpers of the 5th-generation tensor-core kernels (tcgen05, TMEM, mbarriers, bulk copies)
// shared by the thick restart (k_restart_tc.cu) and the Gram-Schmidt pair on tensor cores (k_gs_tc.cu).  Every
// mbarrier wait is bounded by T5_WAIT_LIMIT polls.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"

namespace ksg {

constexpr int T5_WAIT_LIMIT = 1 << 22;

KS_DEVICE uint32_t t5_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor (sm_100 family): start address, leading-dimension byte offset (between core
// matrices adjacent in K), stride byte offset (between 8-row groups), version 1, no swizzle
KS_DEVICE uint64_t t5_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

KS_DEVICE void t5_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

KS_DEVICE void t5_commit(unsigned long long *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(t5_smem(bar))
               : "memory");
}

KS_DEVICE void t5_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
KS_DEVICE void t5_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// bounded wait for the completion of the mbarrier phase with this parity; false on timeout
KS_DEVICE bool t5_wait(unsigned long long *bar, uint32_t parity) {
  const uint32_t a = t5_smem(bar);
  for (int it = 0; it < T5_WAIT_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 16 consecutive TMEM columns of the warp's 32 lanes (one FP32 per thread and column)
KS_DEVICE void t5_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Two signed 7-bit slices as a bf16x2 word, with the encoding of __float2bfloat16_rn(neg ? -(float)u : (float)u)
// (a negative value's zero slice is -0): 0x4300 | u is the bf16 of 128 + u, one exact bf16x2 subtraction of 128
// leaves u, and the sign bits are set after it.  Integer and FMA-pipe operations only.
KS_DEVICE uint32_t t5_slice_pair(uint32_t u0, uint32_t u1, uint32_t neg0, uint32_t neg1) {
  const uint32_t biased = 0x43004300u | u0 | (u1 << 16);
  const __nv_bfloat162 d = __hsub2(*reinterpret_cast<const __nv_bfloat162 *>(&biased),
                                   __floats2bfloat162_rn(128.0f, 128.0f));
  return *reinterpret_cast<const uint32_t *>(&d) | (neg0 << 15) | (neg1 << 31);
}

// the 7-bit field s of a 56-bit magnitude held as (hi, lo) 32-bit halves: bits [49 - 7 s, 56 - 7 s)
KS_DEVICE uint32_t t5_field(uint32_t hi, uint32_t lo, int sl) {
  const int b = 49 - 7 * sl;  // compile-time after unrolling
  if (b >= 32) return (hi >> (b - 32)) & 127u;
  if (b + 7 <= 32) return (lo >> b) & 127u;
  return __funnelshift_r(lo, hi, b) & 127u;
}

KS_DEVICE void t5_expect_tx(unsigned long long *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(t5_smem(bar)), "r"(bytes) : "memory");
}

// global -> shared bulk copy (TMA engine), completion counted in bytes on the mbarrier; 16-byte aligned, size a
// multiple of 16
KS_DEVICE void t5_bulk(void *dst, const void *src, uint32_t bytes, unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(t5_smem(dst)),
      "l"(src), "r"(bytes), "r"(t5_smem(bar))
      : "memory");
}

// 2^k as a double (bit construction in the normal range)
KS_DEVICE double t5_pow2(int k) {
  if (k >= -1022 && k <= 1023) return __longlong_as_double((long long)(1023 + k) << 52);
  return ldexp(1.0, k);
}


}  // namespace ksg
