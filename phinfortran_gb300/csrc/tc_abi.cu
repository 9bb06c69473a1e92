// FP64-grade complex GEMM on tcgen05 (sm_103a): exact BF16 slice products.
//
// Splitting (after Ozaki, Ogita, Oishi and Rump, "Error-free transformations
// of matrix multiplication by using fast routines of matrix multiplication",
// Numer. Algorithms 59, 2012, with integer slices as in Mukunoki, Ozaki,
// Ogita and Imamura, ISC 2020):
//   * the complex product is the real product of the interleaved embeddings
//       Abig(2i, 2j..2j+1) = [Re a_ij, -Im a_ij], Abig(2i+1, ..) = [Im a_ij, Re a_ij]
//       Bbig(c, 2j..2j+1)  = [Re b_jc, Im b_jc]
//     so Cbig = Abig Bbig^T has Re c_ic in row 2i and Im c_ic in row 2i+1 --
//     the interleaved (re, im) order of the complex(kind=8) output;
//   * every row of op(A) (every column of op(B)) is scaled by a power of two
//     2^-e (e: exponent of its largest entry), so |x| < 1, and x*2^63 is
//     truncated to a 63-bit integer F (integer operations on the FP64 bits);
//   * slice s = 1..9 holds q_s * 2^-7s with q_s the s-th 7-bit group of F
//     (|q_s| <= 127: exact in BF16), so x = sum_s q_s 2^-7s + O(2^-63).
//     An entry 2^-10 below the largest of its row still keeps all 53 bits
//     (the blocks of a wide multi-orbital ribbon span several decades);
//   * the product keeps the slice pairs with s + t <= 10.  For s + t <= 7 the
//     FP32 tensor-core sums over K chunks of 256 are integers below 2^22
//     (127^2 * 256 < 2^22), hence exact; each chunk is drained from TMEM and
//     added into a 64-bit fixed-point sum (LSB 2^-49).  The pairs with
//     s + t >= 8 weigh at most 2^-56 and share one FP32 accumulator over the
//     whole K.  The tensor cores' FP32 sums are not correctly rounded: a long
//     inexact chain drifts with a bias (about 2^-24 of the accumulator per
//     MMA), so only light pairs may share it -- with the pairs of sum 7 in
//     it the products were 7 (median) to 64 (maximum) units of 2^-53 |A| |B|
//     away from the exact product on random inputs, against 0.2 to 0.6 for
//     an FP64 GEMM, and a 768-wide ribbon's T moved by 2e-7.
// The result is assembled in FP64 once per output element and scaled back
// by 2^(e_row + e_col).  Relative to |A| |B| the error is O(K 2^-55), the
// accuracy of an FP64 GEMM.
//
// Product kernel: a 128 x 64 output tile of Cbig per CTA (128 threads, two
// CTAs per SM).  Thread 0 issues the TMA loads (cp.async.bulk.tensor, 128-byte
// swizzle, mbarrier completion) of one A slice chunk (128 rows x 256 K) and,
// for each partner slice, one B chunk (64 rows x 256 K), then the
// tcgen05.mma (kind::f16, BF16 in, FP32 accumulate in TMEM) of the pair and
// a tcgen05.commit; all four warps drain the accumulator lanes they own with
// tcgen05.ld.  Every wait is bounded (about a second of clock cycles); a
// wait that gives up sets an error bit, waits once more for what is in
// flight, and the CTA returns after freeing its TMEM.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <mutex>

#include "../../include/phinfortran_gb300.h"
#include "tc_gemm.h"
#include "tc_ptx.cuh"

namespace pf {
namespace tc {
namespace {

constexpr int kThreads = 128;
constexpr int kBoxA = kBM * kKStep * 2;   // bytes of one A box (16 KB)
constexpr int kBoxB = kBN * kKStep * 2;   // bytes of one B box (8 KB)
constexpr int kBoxes = kChunk / kKStep;   // boxes per chunk
constexpr int kSmemA = kBoxes * kBoxA;
constexpr int kSmemB = kBoxes * kBoxB;
constexpr int kSmemBytes = 1024 + kSmemA + kSmemB + 64;
constexpr int kTmemCols = 2 * kBN;        // top slot [0, kBN), low slot [kBN, 2 kBN)

static_assert(kTmemCols >= 32 && (kTmemCols & (kTmemCols - 1)) == 0, "TMEM allocation must be a power of 2");
static_assert(kChunk * 127 * 127 < (1 << 22), "exact chain bound");
static_assert(kSlicesL * kBeta == 63, "63-bit fixed point");
constexpr int kTopDL = 7;  // largest exact pair sum (1-based) of the large products
static_assert(kSlicesL + 1 > kTopDL, "the low accumulator receives at least one pair per chunk");
static_assert(kTopDL * kBeta == 49, "fixed-point LSB used in the epilogue");
// |F| <= chunks * sum_d (d - 1) (127^2 kChunk) 2^(7 (kTopDL - d)): about
// 2^57 a chunk, so at most kMaxChunks chunks (K <= kMaxChunks kChunk real,
// half of it complex) stay below 2^62
constexpr int kMaxChunks = 16;
constexpr double fixed_bound() {
  double b = 0.0, w = 1.0;
  for (int d = kTopDL; d >= 2; --d, w *= 128.0) b += (d - 1) * 127.0 * 127.0 * kChunk * w;
  return b * kMaxChunks;
}
static_assert(fixed_bound() < 4.611686018427388e18, "64-bit fixed-point range (2^62)");
static_assert(2 * kMaxK <= kMaxChunks * kChunk, "K limit of the public entry");

// ---------------------------------------------------------------------------
// TMA tile load (4-D map: K, rows, slice, batch)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5}], [%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}
// ---------------------------------------------------------------------------
// Operands as vector sets: element j of vector v is base[v * sv + j * sj]
// (conjugated when conj).  Rows of op(A) and columns of op(B).
// ---------------------------------------------------------------------------
struct VecSet {
  const double2* base;
  long long sv, sj;
  long long sb;   // batch stride
  bool conj;
  int nvec, len, nbatch;
};

// 32 vectors per block, 8 threads along each (consecutive vectors adjacent
// in memory: a warp reads 32 neighbouring elements per step)
__global__ void vec_exp_thread(VecSet V, const int* active, int* e) {
  const int b = blockIdx.y;
  if (active && !active[b]) return;
  __shared__ unsigned long long red[8][32];
  const int v = blockIdx.x * 32 + threadIdx.x;
  unsigned long long m = 0;
  if (v < V.nvec) {
    const double2* p = V.base + (size_t)b * V.sb + (size_t)v * V.sv;
    for (int j = threadIdx.y; j < V.len; j += 8) {
      const double2 a = p[(size_t)j * V.sj];
      const unsigned long long x = mag_bits(a.x), y = mag_bits(a.y);
      m = x > m ? x : m;
      m = y > m ? y : m;
    }
  }
  red[threadIdx.y][threadIdx.x] = m;
  __syncthreads();
  if (threadIdx.y == 0 && v < V.nvec) {
    for (int k = 1; k < 8; ++k) m = red[k][threadIdx.x] > m ? red[k][threadIdx.x] : m;
    e[(size_t)b * V.nvec + v] = exp_of_maxbits(m);
  }
}
// one warp per vector (contiguous vectors)
__global__ void vec_exp_warp(VecSet V, const int* active, int* e) {
  const int b = blockIdx.y;
  if (active && !active[b]) return;
  const int v = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (v >= V.nvec) return;
  const double2* p = V.base + (size_t)b * V.sb + (size_t)v * V.sv;
  unsigned long long m = 0;
  for (int j = lane; j < V.len; j += 32) {
    const double2 a = p[(size_t)j * V.sj];
    const unsigned long long x = mag_bits(a.x), y = mag_bits(a.y);
    m = x > m ? x : m;
    m = y > m ? y : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, m, o);
    m = w > m ? w : m;
  }
  if (lane == 0) e[(size_t)b * V.nvec + v] = exp_of_maxbits(m);
}

// Slices of a vector set into out[b][s][row][kp] (BF16, K-major rows).
// pair = true: two rows per vector (the A embedding: 2v -> [re, -im],
// 2v+1 -> [im, re]); pair = false: one row per vector ([re, im]).
// One thread per (vector, complex index j); indices j >= len write zeros
// up to kp / 2.
__global__ void vec_slice(VecSet V, const int* active, const int* e, int kp, bool pair, uint16_t* out) {
  const int b = blockIdx.z;
  if (active && !active[b]) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int v = blockIdx.y * blockDim.y + threadIdx.y;
  if (v >= V.nvec || 2 * j >= kp) return;
  const int rows = pair ? 2 * V.nvec : V.nvec;
  double2 a = make_double2(0.0, 0.0);
  const int ev = e[(size_t)b * V.nvec + v];
  if (j < V.len) {
    a = V.base[(size_t)b * V.sb + (size_t)v * V.sv + (size_t)j * V.sj];
    if (V.conj) a.y = -a.y;
  }
  bool nre, nim;
  const unsigned long long Fr = fixed_pt<kSlicesL * kBeta>(a.x, ev, nre);
  const unsigned long long Fi = fixed_pt<kSlicesL * kBeta>(a.y, ev, nim);
#pragma unroll
  for (int s = 1; s <= kSlicesL; ++s) {
    const uint16_t re = slice_bf16_n<kSlicesL>(Fr, s, nre);
    const uint16_t im = slice_bf16_n<kSlicesL>(Fi, s, nim);
    const size_t plane = ((size_t)b * kSlicesL + (s - 1)) * rows;
    if (pair) {
      const uint16_t mim = im ? (uint16_t)(im ^ 0x8000u) : (uint16_t)0;
      uint32_t* r0 = reinterpret_cast<uint32_t*>(out + (plane + 2 * (size_t)v) * kp + 2 * j);
      uint32_t* r1 = reinterpret_cast<uint32_t*>(out + (plane + 2 * (size_t)v + 1) * kp + 2 * j);
      *r0 = (uint32_t)re | ((uint32_t)mim << 16);
      *r1 = (uint32_t)im | ((uint32_t)re << 16);
    } else {
      uint32_t* r0 = reinterpret_cast<uint32_t*>(out + (plane + (size_t)v) * kp + 2 * j);
      *r0 = (uint32_t)re | ((uint32_t)im << 16);
    }
  }
}

// ---------------------------------------------------------------------------
// Product kernel
// ---------------------------------------------------------------------------
struct ProdArgs {
  int m, n, kp;              // complex m (Cbig has 2m rows), n, padded real K
  int a_shared, b_shared;
  const int* ea;             // [nbA][m]
  const int* eb;             // [nbB][n]
  double* C;                 // interleaved complex
  int ldc;
  long long sC;
  double alpha, beta;
  const int* active;
  const double2* zdiag;
  const double* H;
  int ldh;
  long long sH;
  int* err;
};

__global__ void __launch_bounds__(kThreads, 2)
    tc_prod_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, ProdArgs p) {
  const int b = blockIdx.z;
  if (p.active && !p.active[b]) return;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                         ~(uintptr_t)1023);
  unsigned char* sA = smem;
  unsigned char* sB = smem + kSmemA;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sB + kSmemB);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + 4);
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t bar_a = smem_u32(&bars[0]), bar_b = smem_u32(&bars[1]), bar_m = smem_u32(&bars[2]);
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
  const int ba = p.a_shared ? 0 : b, bb = p.b_shared ? 0 : b;

  if (tid == 0) {
    mbar_init(bar_a, 1);
    mbar_init(bar_b, 1);
    mbar_init(bar_m, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
  constexpr uint32_t idesc = idesc_bf16(kBM, kBN);

  long long F[kBN];
#pragma unroll
  for (int j = 0; j < kBN; ++j) F[j] = 0;
  uint32_t ph_a = 0, ph_b = 0, ph_m = 0;
  bool low_init = false;               // thread 0: the low accumulator holds a value
  bool abort = false;
  uint32_t pend_bar = 0, pend_ph = 0;  // the wait that gave up
  const int nchunk = (p.kp + kChunk - 1) / kChunk;
  for (int c = 0; c < nchunk && !abort; ++c) {
    const int k0 = c * kChunk;
    const int ks = min(kBoxes, (p.kp - k0) / kKStep);
    for (int s = 0; s < kSlicesL && !abort; ++s) {
      if (tid == 0) {
        mbar_expect_tx(bar_a, (uint32_t)(ks * kBoxA));
        for (int u = 0; u < ks; ++u) tma_load_4d(smem_u32(sA + u * kBoxA), &ta, k0 + u * kKStep, m0, s, ba, bar_a);
      }
      abort = __syncthreads_or(!mbar_wait(bar_a, ph_a));
      pend_bar = bar_a;
      pend_ph = ph_a;
      ph_a ^= 1;
      for (int t = 0; s + t <= kSlicesL - 1 && !abort; ++t) {
        const int d = s + t + 2;  // 1-based pair sum
        const bool top = d <= kTopDL;
        if (tid == 0) {
          mbar_expect_tx(bar_b, (uint32_t)(ks * kBoxB));
          for (int u = 0; u < ks; ++u)
            tma_load_4d(smem_u32(sB + u * kBoxB), &tb, k0 + u * kKStep, n0, t, bb, bar_b);
        }
        abort = __syncthreads_or(!mbar_wait(bar_b, ph_b));
        pend_bar = bar_b;
        pend_ph = ph_b;
        ph_b ^= 1;
        if (abort) break;
        if (tid == 0) {
          tc_fence_after();
          const uint32_t dcol = top ? 0u : (uint32_t)kBN;
          for (int u = 0; u < ks; ++u) {
#pragma unroll
            for (int kk = 0; kk < kKStep / 16; ++kk) {
              const uint64_t ad = desc_sw128(smem_u32(sA + u * kBoxA + kk * 32));
              const uint64_t bd = desc_sw128(smem_u32(sB + u * kBoxB + kk * 32));
              const uint32_t acc = top ? (uint32_t)((u | kk) != 0) : (uint32_t)(low_init || (u | kk) != 0);
              mma_bf16(tmem + dcol, ad, bd, idesc, acc);
            }
          }
          if (!top) low_init = true;
          mma_commit(bar_m);
        }
        abort = __syncthreads_or(!mbar_wait(bar_m, ph_m));
        pend_bar = bar_m;
        pend_ph = ph_m;
        ph_m ^= 1;
        if (abort) break;
        tc_fence_after();
        if (top) {
          // exact integer partial sums: I = v 2^(7d), |I| < 2^22
          const float scale = __int_as_float((127 + kBeta * d) << 23);
          const int sh = kBeta * (kTopDL - d);
#pragma unroll
          for (int q = 0; q < kBN / 16; ++q) {
            uint32_t r[16];
            tmem_ld16(lane_base + q * 16, r);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const float f = fmaf(__uint_as_float(r[j]), scale, 12582912.0f);
              const int I = __float_as_int(f) - 0x4B400000;
              F[q * 16 + j] += (long long)I << sh;
            }
          }
        }
        tc_fence_before();
        __syncthreads();
      }
    }
  }
  if (abort) {
    // give the copies or products still in flight one more bounded wait
    // before the shared memory and TMEM are released
    (void)mbar_wait(pend_bar, pend_ph);
    if (tid == 0 && p.err) atomicOr(p.err, 1);
  } else {
    tc_fence_after();
    const int R = m0 + tid;  // row of Cbig owned by this thread (TMEM lane)
    const bool rowok = R < 2 * p.m;
    const int i = R >> 1, part = R & 1;
    const int ea = rowok ? p.ea[(size_t)ba * p.m + i] : 0;
    double* Cb = p.C + (size_t)b * p.sC * 2;
#pragma unroll
    for (int q = 0; q < kBN / 16; ++q) {
      uint32_t r[16];
      tmem_ld16(lane_base + kBN + q * 16, r);  // every chunk has low pairs: the slot is written
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int col = n0 + q * 16 + j;
        if (!rowok || col >= p.n) continue;
        const int eb = p.eb[(size_t)bb * p.n + col];
        double v;
        if (ea == kExpBad || eb == kExpBad) {
          v = __longlong_as_double(0x7FF8000000000000ll);
        } else {
          const double top = (double)F[q * 16 + j] * 0x1p-49;  // LSB 2^(-7 kTopDL)
          v = scalbn(top + (double)__uint_as_float(r[j]), ea + eb);
        }
        v *= p.alpha;
        const size_t at = 2 * ((size_t)i + (size_t)col * p.ldc) + part;
        if (p.beta != 0.0) v = fma(p.beta, Cb[at], v);
        if (p.H) v -= p.H[(size_t)b * p.sH * 2 + 2 * ((size_t)i + (size_t)col * p.ldh) + part];
        if (p.zdiag && i == col) v += part ? p.zdiag[b].y : p.zdiag[b].x;
        Cb[at] = v;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

// ---------------------------------------------------------------------------
// Pipelined product kernel: the same tile and arithmetic as tc_prod_kernel,
// with warp roles and double buffering so that loads, products and drains
// overlap.  192 threads: warp 0 issues the TMA loads, warp 1 the tcgen05.mma
// (one elected lane each), warps 2..5 drain TMEM (warp w reads lanes
// 32 (w mod 4) .. +31) and write C.  Shared memory: two A chunks (128 rows x
// 256 K) and two B chunks (64 rows x 256 K); TMEM: two accumulators for the
// exact pairs (drained while the next pair accumulates) and the low slot.
// Job order, identical in every role: chunk c, slice s of A, slice t of B.
// Every wait is bounded and also gives up when another role has given up.
// ---------------------------------------------------------------------------
constexpr int kPipeThreads = 192;
constexpr int kPipeTmemCols = 256;   // top slots [0, 64), [64, 128); low [128, 192)
constexpr int kPipeSmem = 1024 + 2 * kSmemA + 2 * kSmemB + 256;
static_assert(3 * kBN <= kPipeTmemCols, "TMEM slots");

enum { BA_FULL = 0, BA_EMPTY = 2, BB_FULL = 4, BB_EMPTY = 6, BACC_FULL = 8, BACC_EMPTY = 10, BLOW = 12, BFIN = 13,
       NBAR = 14 };

// Bounded wait that also returns false once *abort is set; a wait that runs
// out of time sets *abort itself.
__device__ __forceinline__ bool mbar_wait_ab(uint32_t bar, uint32_t parity, volatile int* abort) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t done = 0;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (*abort) return false;
    if (clock64() - t0 > kWaitCycles) {
      *abort = 1;
      return false;
    }
  }
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__global__ void __launch_bounds__(kPipeThreads, 1)
    tc_prod_pipe_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, ProdArgs p) {
  const int b = blockIdx.z;
  if (p.active && !p.active[b]) return;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                         ~(uintptr_t)1023);
  unsigned char* sA = smem;                   // 2 stages of kSmemA
  unsigned char* sB = smem + 2 * kSmemA;      // 2 stages of kSmemB
  uint64_t* bars = reinterpret_cast<uint64_t*>(sB + 2 * kSmemB);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + NBAR);
  volatile int* abort = reinterpret_cast<volatile int*>(tmem_holder + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
  const int ba = p.a_shared ? 0 : b, bb = p.b_shared ? 0 : b;
  auto bar = [&](int i) { return smem_u32(&bars[i]); };

  if (tid == 0) {
    for (int i = 0; i < NBAR; ++i) mbar_init(bar(i), (i == BACC_EMPTY || i == BACC_EMPTY + 1) ? 4u : 1u);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                 "r"(kPipeTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  const int nchunk = (p.kp + kChunk - 1) / kChunk;

  if (warp == 0) {
    // ---- TMA producer
    if (lane == 0) {
      int ja = 0, jb = 0;
      uint32_t last_a = 0, last_a_ph = 0, last_b = 0, last_b_ph = 0;
      bool ok = true;
      for (int c = 0; c < nchunk && ok; ++c) {
        const int k0 = c * kChunk;
        const int ks = min(kBoxes, (p.kp - k0) / kKStep);
        for (int s = 0; s < kSlicesL && ok; ++s) {
          const int as = ja & 1, ka = ja >> 1;
          if (!(ok = mbar_wait_ab(bar(BA_EMPTY + as), (ka & 1) ^ 1, abort))) break;
          mbar_expect_tx(bar(BA_FULL + as), (uint32_t)(ks * kBoxA));
          for (int u = 0; u < ks; ++u)
            tma_load_4d(smem_u32(sA + as * kSmemA + u * kBoxA), &ta, k0 + u * kKStep, m0, s, ba, bar(BA_FULL + as));
          last_a = bar(BA_FULL + as);
          last_a_ph = ka & 1;
          ++ja;
          for (int t = 0; s + t <= kSlicesL - 1; ++t) {
            const int bs = jb & 1, kb = jb >> 1;
            if (!(ok = mbar_wait_ab(bar(BB_EMPTY + bs), (kb & 1) ^ 1, abort))) break;
            mbar_expect_tx(bar(BB_FULL + bs), (uint32_t)(ks * kBoxB));
            for (int u = 0; u < ks; ++u)
              tma_load_4d(smem_u32(sB + bs * kSmemB + u * kBoxB), &tb, k0 + u * kKStep, n0, t, bb,
                          bar(BB_FULL + bs));
            last_b = bar(BB_FULL + bs);
            last_b_ph = kb & 1;
            ++jb;
          }
        }
      }
      if (!ok) {
        // copies still in flight land before the CTA's shared memory is released
        if (last_a) (void)mbar_wait(last_a, last_a_ph);
        if (last_b) (void)mbar_wait(last_b, last_b_ph);
      }
    }
  } else if (warp == 1) {
    // ---- MMA issuer
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(kBM, kBN);
      int ja = 0, jb = 0, jt = 0;
      bool low_init = false, ok = true;
      for (int c = 0; c < nchunk && ok; ++c) {
        const int k0 = c * kChunk;
        const int ks = min(kBoxes, (p.kp - k0) / kKStep);
        for (int s = 0; s < kSlicesL && ok; ++s) {
          const int as = ja & 1, ka = ja >> 1;
          if (!(ok = mbar_wait_ab(bar(BA_FULL + as), ka & 1, abort))) break;
          for (int t = 0; s + t <= kSlicesL - 1; ++t) {
            const int d = s + t + 2;
            const bool top = d <= kTopDL;
            const int bs = jb & 1, kb = jb >> 1;
            if (!(ok = mbar_wait_ab(bar(BB_FULL + bs), kb & 1, abort))) break;
            const int slot = jt & 1, kt = jt >> 1;
            if (top && !(ok = mbar_wait_ab(bar(BACC_EMPTY + slot), (kt & 1) ^ 1, abort))) break;
            tc_fence_after();
            const uint32_t dcol = top ? (uint32_t)(slot * kBN) : (uint32_t)(2 * kBN);
            for (int u = 0; u < ks; ++u) {
#pragma unroll
              for (int kk = 0; kk < kKStep / 16; ++kk) {
                const uint64_t ad = desc_sw128(smem_u32(sA + as * kSmemA + u * kBoxA + kk * 32));
                const uint64_t bd = desc_sw128(smem_u32(sB + bs * kSmemB + u * kBoxB + kk * 32));
                const uint32_t acc = top ? (uint32_t)((u | kk) != 0) : (uint32_t)(low_init || (u | kk) != 0);
                mma_bf16(tmem + dcol, ad, bd, idesc, acc);
              }
            }
            if (!top) low_init = true;
            mma_commit(bar(BB_EMPTY + bs));
            if (top) {
              mma_commit(bar(BACC_FULL + slot));
              ++jt;
            }
            if (s + t == kSlicesL - 1) mma_commit(bar(BA_EMPTY + as));
            ++jb;
          }
          ++ja;
        }
      }
      if (ok) mma_commit(bar(BLOW));
      mma_commit(bar(BFIN));  // arrives once every product issued here has completed
    }
  } else {
    // ---- epilogue: drains of the exact pairs, then the output tile
    const int sub = warp & 3;  // TMEM lane quarter of this warp
    const uint32_t lane_base = tmem + ((uint32_t)(sub * 32) << 16);
    long long F[kBN];
#pragma unroll
    for (int j = 0; j < kBN; ++j) F[j] = 0;
    int jt = 0;
    bool ok = true;
    for (int c = 0; c < nchunk && ok; ++c) {
      for (int s = 0; s < kSlicesL && ok; ++s) {
        for (int t = 0; s + t <= kSlicesL - 1 && ok; ++t) {
          const int d = s + t + 2;
          if (d > kTopDL) continue;
          const int slot = jt & 1, kt = jt >> 1;
          ok = __all_sync(0xffffffffu, mbar_wait_ab(bar(BACC_FULL + slot), kt & 1, abort));
          if (!ok) break;
          tc_fence_after();
          const float scale = __int_as_float((127 + kBeta * d) << 23);
          const int sh = kBeta * (kTopDL - d);
#pragma unroll
          for (int q = 0; q < kBN / 16; ++q) {
            uint32_t r[16];
            tmem_ld16(lane_base + slot * kBN + q * 16, r);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const float f = fmaf(__uint_as_float(r[j]), scale, 12582912.0f);
              const int I = __float_as_int(f) - 0x4B400000;
              F[q * 16 + j] += (long long)I << sh;
            }
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(bar(BACC_EMPTY + slot));
          ++jt;
        }
      }
    }
    if (ok) ok = mbar_wait_ab(bar(BLOW), 0, abort);
    ok = __all_sync(0xffffffffu, ok);
    if (ok) {
      tc_fence_after();
      const int R = m0 + sub * 32 + lane;
      const bool rowok = R < 2 * p.m;
      const int i = R >> 1, part = R & 1;
      const int ea = rowok ? p.ea[(size_t)ba * p.m + i] : 0;
      double* Cb = p.C + (size_t)b * p.sC * 2;
#pragma unroll
      for (int q = 0; q < kBN / 16; ++q) {
        uint32_t r[16];
        tmem_ld16(lane_base + 2 * kBN + q * 16, r);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = n0 + q * 16 + j;
          if (!rowok || col >= p.n) continue;
          const int eb = p.eb[(size_t)bb * p.n + col];
          double v;
          if (ea == kExpBad || eb == kExpBad) {
            v = __longlong_as_double(0x7FF8000000000000ll);
          } else {
            const double top = (double)F[q * 16 + j] * 0x1p-49;  // LSB 2^(-7 kTopDL)
            v = scalbn(top + (double)__uint_as_float(r[j]), ea + eb);
          }
          v *= p.alpha;
          const size_t at = 2 * ((size_t)i + (size_t)col * p.ldc) + part;
          if (p.beta != 0.0) v = fma(p.beta, Cb[at], v);
          if (p.H) v -= p.H[(size_t)b * p.sH * 2 + 2 * ((size_t)i + (size_t)col * p.ldh) + part];
          if (p.zdiag && i == col) v += part ? p.zdiag[b].y : p.zdiag[b].x;
          Cb[at] = v;
        }
      }
    }
  }
  __syncthreads();
  // every product has completed before TMEM is released
  (void)mbar_wait(bar(BFIN), 0);
  if (tid == 0 && *abort && p.err) atomicOr(p.err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kPipeTmemCols));
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn g_encode = nullptr;
bool g_pipe = true;  // pipelined product kernel (false: the synchronous one)
std::once_flag g_encode_once;

void load_encode() {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
          cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    g_encode = reinterpret_cast<EncodeTiledFn>(fn);
  else
    (void)cudaGetLastError();
}

inline size_t r256(size_t x) { return (x + 255) & ~(size_t)255; }
inline int kpad(int k) { return ((2 * k + kKStep - 1) / kKStep) * kKStep; }

// 4-D map over slices [nb][kSlicesL][rows][kp] (BF16) with a box of
// kKStep x box_rows x 1 x 1 and 128-byte swizzling; rows beyond `rows`
// read as zeros
bool encode_slices(CUtensorMap* map, void* base, int kp, int rows, int nb, int box_rows) {
  const cuuint64_t dims[4] = {(cuuint64_t)kp, (cuuint64_t)rows, (cuuint64_t)kSlicesL, (cuuint64_t)nb};
  const cuuint64_t strides[3] = {(cuuint64_t)kp * 2, (cuuint64_t)kp * 2 * rows,
                                 (cuuint64_t)kp * 2 * rows * kSlicesL};
  const cuuint32_t box[4] = {(cuuint32_t)kKStep, (cuuint32_t)box_rows, 1, 1};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return g_encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, base, dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct Carve {
  uint16_t* sa;
  uint16_t* sb;
  int* ea;
  int* eb;
  size_t bytes;
};
Carve carve(char* base, int m, int n, int k, int nba, int nbb) {
  const int kp = kpad(k);
  Carve c;
  size_t off = 0;
  const size_t a_b = r256((size_t)nba * kSlicesL * 2 * m * kp * 2);
  const size_t b_b = r256((size_t)nbb * kSlicesL * n * kp * 2);
  c.sa = reinterpret_cast<uint16_t*>(base ? base + off : nullptr);
  off += a_b;
  c.sb = reinterpret_cast<uint16_t*>(base ? base + off : nullptr);
  off += b_b;
  c.ea = reinterpret_cast<int*>(base ? base + off : nullptr);
  off += r256((size_t)nba * m * 4);
  c.eb = reinterpret_cast<int*>(base ? base + off : nullptr);
  off += r256((size_t)nbb * n * 4);
  c.bytes = off;
  return c;
}

void launch_exp(const VecSet& V, const int* active, int* e, cudaStream_t st) {
  if (V.sv == 1)
    vec_exp_thread<<<dim3((V.nvec + 31) / 32, V.nbatch), dim3(32, 8), 0, st>>>(V, active, e);
  else
    vec_exp_warp<<<dim3((V.nvec + 7) / 8, V.nbatch), 256, 0, st>>>(V, active, e);
}
void launch_slice(const VecSet& V, const int* active, const int* e, int kp, bool pair, uint16_t* out,
                  cudaStream_t st) {
  const dim3 blk(64, 4);
  const dim3 grid((kp / 2 + 63) / 64, (V.nvec + 3) / 4, V.nbatch);
  vec_slice<<<grid, blk, 0, st>>>(V, active, e, kp, pair, out);
}

}  // namespace

bool tma_available() {
  std::call_once(g_encode_once, load_encode);
  return g_encode != nullptr;
}

size_t zgemm_workspace(int m, int n, int k, int batch, bool a_shared, bool b_shared) {
  if (m <= 0 || n <= 0 || k <= 0 || batch <= 0) return 0;
  return carve(nullptr, m, n, k, a_shared ? 1 : batch, b_shared ? 1 : batch).bytes;
}

cudaError_t zgemm(const ZgemmArgs& g, void* work, size_t work_bytes, int* err, cudaStream_t st) {
  if (g.m <= 0 || g.n <= 0 || g.batch <= 0) return cudaSuccess;
  if (g.k <= 0 || g.k > kMaxK) return cudaErrorInvalidValue;
  if (!tma_available()) return cudaErrorNotSupported;
  const bool ash = g.sA == 0, bsh = g.sB == 0;
  const int nba = ash ? 1 : g.batch, nbb = bsh ? 1 : g.batch;
  const int kp = kpad(g.k);
  Carve c = carve(reinterpret_cast<char*>(work), g.m, g.n, g.k, nba, nbb);
  if (!work || work_bytes < c.bytes) return cudaErrorInvalidValue;
  const double2* A = reinterpret_cast<const double2*>(g.A);
  const double2* B = reinterpret_cast<const double2*>(g.B);
  // rows of op(A): element (i, j) = A[i + j lda] or conj(A[j + i lda])
  VecSet va{A, g.ca ? (long long)g.lda : 1, g.ca ? 1 : (long long)g.lda, ash ? 0 : g.sA, g.ca, g.m, g.k, nba};
  // columns of op(B): element (j, c) = B[j + c ldb] or conj(B[c + j ldb])
  VecSet vb{B, g.cb ? 1 : (long long)g.ldb, g.cb ? (long long)g.ldb : 1, bsh ? 0 : g.sB, g.cb, g.n, g.k, nbb};
  // shared operands are prepared for every element (no mask); per-point ones skip retired points
  const int* ma = ash ? nullptr : g.active;
  const int* mb = bsh ? nullptr : g.active;
  launch_exp(va, ma, c.ea, st);
  launch_exp(vb, mb, c.eb, st);
  launch_slice(va, ma, c.ea, kp, true, c.sa, st);
  launch_slice(vb, mb, c.eb, kp, false, c.sb, st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  CUtensorMap ta, tb;
  if (!encode_slices(&ta, c.sa, kp, 2 * g.m, nba, kBM) || !encode_slices(&tb, c.sb, kp, g.n, nbb, kBN))
    return cudaErrorInvalidValue;
  ProdArgs p;
  p.m = g.m;
  p.n = g.n;
  p.kp = kp;
  p.a_shared = ash;
  p.b_shared = bsh;
  p.ea = c.ea;
  p.eb = c.eb;
  p.C = reinterpret_cast<double*>(g.C);
  p.ldc = g.ldc;
  p.sC = g.sC;
  p.alpha = g.alpha;
  p.beta = g.beta;
  p.active = g.active;
  p.zdiag = reinterpret_cast<const double2*>(g.zdiag);
  p.H = reinterpret_cast<const double*>(g.H);
  p.ldh = g.ldh;
  p.sH = g.sH;
  p.err = err;
  const dim3 grid((2 * g.m + kBM - 1) / kBM, (g.n + kBN - 1) / kBN, g.batch);
  if (g_pipe) {
    e = cudaFuncSetAttribute(tc_prod_pipe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPipeSmem);
    if (e != cudaSuccess) return e;
    tc_prod_pipe_kernel<<<grid, kPipeThreads, kPipeSmem, st>>>(ta, tb, p);
  } else {
    e = cudaFuncSetAttribute(tc_prod_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) return e;
    tc_prod_kernel<<<grid, kThreads, kSmemBytes, st>>>(ta, tb, p);
  }
  return cudaGetLastError();
}

}  // namespace tc
}  // namespace pf

// ---------------------------------------------------------------------------
// extern "C" entry: batched FP64-grade complex GEMM
// ---------------------------------------------------------------------------
namespace {
thread_local char g_tc_err[256] = "";
int tc_set_err(int code, const char* msg) {
  snprintf(g_tc_err, sizeof(g_tc_err), "%s", msg);
  return code;
}
}  // namespace

extern "C" {

const char* pf_tc_last_error(void) { return g_tc_err; }

size_t pf_tc_zgemm_workspace_size(int m, int n, int k, int batch, int a_shared, int b_shared) {
  const size_t w = pf::tc::zgemm_workspace(m, n, k, batch, a_shared != 0, b_shared != 0);
  return w ? w + 256 : 0;
}

int pf_tc_zgemm_dev(int transa, int transb, int m, int n, int k, double alpha, const double* A, int lda,
                    long long strideA, const double* B, int ldb, long long strideB, double beta, double* C, int ldc,
                    long long strideC, int batch, void* work, size_t work_bytes, void* stream) {
  if (m < 0 || n < 0 || k < 0 || batch < 0) return tc_set_err(PF_ERR_ARG, "pf_tc_zgemm: negative size");
  if ((transa != 'N' && transa != 'C') || (transb != 'N' && transb != 'C'))
    return tc_set_err(PF_ERR_ARG, "pf_tc_zgemm: trans must be 'N' or 'C'");
  if (m == 0 || n == 0 || batch == 0) return PF_SUCCESS;
  if (k == 0) return tc_set_err(PF_ERR_ARG, "pf_tc_zgemm: k must be positive");
  if (k > pf::tc::kMaxK) return tc_set_err(PF_ERR_SIZE, "pf_tc_zgemm: k above 2048");
  if (!A || !B || !C || !work) return tc_set_err(PF_ERR_ARG, "pf_tc_zgemm: null pointer");
  const int rowsA = transa == 'N' ? m : k, rowsB = transb == 'N' ? k : n;
  if (lda < rowsA || ldb < rowsB || ldc < m) return tc_set_err(PF_ERR_ARG, "pf_tc_zgemm: leading dimension too small");
  const size_t need = pf_tc_zgemm_workspace_size(m, n, k, batch, strideA == 0, strideB == 0);
  if (work_bytes < need) return tc_set_err(PF_ERR_ARG, "pf_tc_zgemm: workspace too small");
  if (!pf::tc::tma_available()) return tc_set_err(PF_ERR_CUDA, "pf_tc_zgemm: cuTensorMapEncodeTiled unavailable");
  char* w = reinterpret_cast<char*>(work);
  int* err = reinterpret_cast<int*>(w);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), st);
  if (e != cudaSuccess) return tc_set_err(PF_ERR_CUDA, cudaGetErrorString(e));
  pf::tc::ZgemmArgs g{};
  g.m = m;
  g.n = n;
  g.k = k;
  g.A = A;
  g.lda = lda;
  g.sA = strideA;
  g.ca = transa == 'C';
  g.B = B;
  g.ldb = ldb;
  g.sB = strideB;
  g.cb = transb == 'C';
  g.C = C;
  g.ldc = ldc;
  g.sC = strideC;
  g.alpha = alpha;
  g.beta = beta;
  g.batch = batch;
  e = pf::tc::zgemm(g, w + 256, work_bytes - 256, err, st);
  if (e != cudaSuccess) return tc_set_err(PF_ERR_CUDA, cudaGetErrorString(e));
  int herr = 0;
  e = cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return tc_set_err(PF_ERR_CUDA, cudaGetErrorString(e));
  if (herr) return tc_set_err(PF_ERR_CUDA, "pf_tc_zgemm: a pipeline wait of the product kernel timed out");
  return PF_SUCCESS;
}

}  // extern "C"
