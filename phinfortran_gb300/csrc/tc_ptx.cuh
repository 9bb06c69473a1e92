// PTX wrappers and the slice arithmetic shared by the tensor-core GEMMs
// (tc_abi.cu: batched large products fed by TMA; mixed.cuh: the 32-wide
// lead decimations, operands sliced by the CTA into shared memory).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tc_gemm.h"

namespace pf {
namespace tc {

constexpr int kExpBad = -100000;          // exponent marker of a non-finite vector
constexpr long long kWaitCycles = 1LL << 31;  // bound of every mbarrier wait (~1 s)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Bounded wait for the phase with the given parity; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > kWaitCycles) return false;
  }
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor (sm_100 format) of a K-major operand tile
// written by TMA with 128-byte swizzling: rows of 128 bytes, 8-row groups
// 1024 bytes apart (stride byte offset), layout type 2 = SWIZZLE_128B,
// descriptor version 1 in bits 46-47.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;              // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset
  d |= (uint64_t)1 << 46;              // version
  d |= (uint64_t)2 << 61;              // SWIZZLE_128B
  return d;
}
// Instruction descriptor of kind::f16: D = FP32 (bits 4-5 = 1), A = B = BF16
// (bits 7-9, 10-12 = 1), both K-major, N >> 3 in bits 17-22, M >> 4 in 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}

// The same load without the wait: several loads are issued back to back and
// completed by one tmem_wait_ld() before any of their registers is used.
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// Ties registers filled by tmem_ld16_nowait to a point after tmem_wait_ld():
// the compiler sees them redefined here (volatile asm statements keep their
// order), so no use of them moves above the wait.
__device__ __forceinline__ void tmem_regs_ready(uint32_t (&r)[16]) {
  asm volatile(""
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15]));
}

__device__ __forceinline__ unsigned long long mag_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
}
// exponent e with max|.| < 2^e (0 for an all-zero vector, kExpBad when a
// component is not finite), from the largest magnitude's bit pattern
__device__ __forceinline__ int exp_of_maxbits(unsigned long long m) {
  const int ef = (int)(m >> 52);
  if (ef == 0x7FF) return kExpBad;
  if (m == 0) return 0;
  return ef == 0 ? -1022 : ef - 1022;
}

// Bits-bit truncated fixed point of x = a 2^-e (|x| < 1), from the FP64
// bits (integer operations only); the sign is returned separately.
template <int Bits>
__device__ __forceinline__ unsigned long long fixed_pt(double a, int e, bool& neg) {
  static_assert(Bits >= 53 && Bits <= 63, "one 64-bit word");
  const unsigned long long bits = (unsigned long long)__double_as_longlong(a);
  neg = (bits >> 63) != 0;
  const int ef = (int)((bits >> 52) & 0x7FF);
  unsigned long long mant = bits & 0x000FFFFFFFFFFFFFull;
  if (ef != 0) mant |= 0x0010000000000000ull;
  if (mant == 0 || e == kExpBad || ef == 0x7FF) return 0;
  const int eeff = ef == 0 ? 1 : ef;
  // a = mant 2^(eeff - 1075); x 2^Bits = mant 2^(eeff - 1075 + Bits - e)
  const int sh = eeff - (1075 - Bits) - e;
  if (sh >= 0) return sh > Bits - 53 ? 0 : (mant << sh);  // sh <= Bits - 53 whenever |x| < 1
  return sh <= -64 ? 0 : (mant >> (-sh));
}
__device__ __forceinline__ unsigned long long fixed56(double a, int e, bool& neg) { return fixed_pt<56>(a, e, neg); }

// BF16 bits of q 2^-(7s), q the s-th 7-bit group (from the top) of the
// (7 Slices)-bit fixed point F
template <int Slices>
__device__ __forceinline__ uint16_t slice_bf16_n(unsigned long long F, int s, bool neg) {
  const int q = (int)((F >> (kBeta * (Slices - s))) & 127u);
  if (q == 0) return 0;
  // q as a float (exact), scaled by 2^-(7s) through the exponent field
  const float f = __int_as_float(0x4B000000 | q) - 8388608.0f;
  const unsigned int fb = (unsigned int)__float_as_int(f) - ((unsigned int)(kBeta * s) << 23);
  return (uint16_t)((fb >> 16) | (neg ? 0x8000u : 0u));
}
__device__ __forceinline__ uint16_t slice_bf16(unsigned long long F, int s, bool neg) {
  return slice_bf16_n<kSlices>(F, s, neg);
}


}  // namespace tc
}  // namespace pf
