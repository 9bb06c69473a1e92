// CTA-level FP64-grade complex products of blocks up to 32 x 32 on tcgen05,
// for the lead decimations of the 32-wide mixed pipeline (the batched
// large products are in tc_abi.cu; the splitting is the same: every row of
// op(A) and column of op(B) scaled by a power of two and cut into eight
// 7-bit BF16 slices, slice pairs with s + t <= 6 summed exactly, the lighter
// ones in one FP32 accumulator, the result assembled in FP64).
//
// One call forms C_kb = op(A_k) op(B_b) for k = 0, 1 and b < NB: the two
// left operands stacked in M (rows 0 .. 2m-1 and 64 .. 64+2m-1 of the
// M = 128 tile), NB = 1 or 2 right operands side by side in N (N = 32 NB).
//
// Layout: the CTA writes the slices itself into shared memory, in the
// K-major 128-byte-swizzled layout that the tcgen05 descriptors read (row r
// of a tile at r * 128 bytes, its 16-byte chunk c stored at chunk c ^ (r & 7)).
// A_big (2m x 2m, the interleaved real embedding of op(A)) fills a 128-row
// tile, B_big (m x 2m per right operand) rows 32 b .. 32 b + m - 1 of a
// 64-row tile; K = 2m <= 64 is one swizzle row.
//
// TMEM: one accumulator of 64 columns per pair sum for the exact pairs
// (sums 2..5, and two for sum 6, so that every exact accumulator stays
// below 2^22 units: 4 pairs x 64 terms x 127^2 < 2^22) and one for the
// light pairs: 7 x 64 of the 512 columns (the kernel runs one CTA per SM).
// All 36 pair products of a call are issued at once (B slices all
// resident, A slices double-buffered), then drained by the eight warps.
//
// Every operand element is read once: the 256 threads hold their elements
// of the two stacked A blocks (8 each) and of the B blocks (4 each per
// block) in registers, find the row / column maxima with shared-memory
// atomics on the high words of the magnitudes, convert to fixed point once
// and cut the slices from registers.
#pragma once
#include "cmat.cuh"
#include "tc_ptx.cuh"

namespace pf {
namespace tc {

constexpr int kSmallN = 32;                            // largest block
constexpr int kSmallNB = 2;                            // most right operands a call
constexpr int kSmallATile = 128 * 128;                 // bytes of one A slice tile
constexpr int kSmallBTile = kSmallNB * kSmallN * 128;  // bytes of one B slice tile
constexpr int kSmallTmemCols = 512;
constexpr int kSmallSlotCols = kSmallNB * kSmallN;     // TMEM columns a slot
constexpr int kSmallExact = 6;                         // exact slots
constexpr int kSmallLow = 6;                           // TMEM slot of the light pairs
constexpr int kSmallThreads = 256;                     // the CTA size small_zgemm is written for
constexpr int kSmallPerA = 2 * kSmallN * kSmallN / kSmallThreads;  // A elements a thread
constexpr int kSmallPerB = kSmallN * kSmallN / kSmallThreads;      // B elements a thread, per block
constexpr int kSmallSmem = 2 * kSmallATile + kSlices * kSmallBTile + (64 + 64) * 4 + 64 + 128 * 4;
static_assert((kSmallLow + 1) * kSmallSlotCols <= kSmallTmemCols, "TMEM slots");
static_assert(kTopD == 6, "slot map of small_slot");

// TMEM slot of the pair (s, t) (0-based slices): pair sums s + t + 2 = 2..5
// have one slot each, sum 6 two (s <= 2 and s >= 3), lighter pairs the low slot
__device__ __forceinline__ int small_slot(int s, int t) {
  const int d = s + t;
  if (d <= 3) return d;
  if (d == 4) return s <= 2 ? 4 : 5;
  return kSmallLow;
}

struct SmallTC {
  unsigned char* a_tile;  // 2 tiles, 1024-aligned
  unsigned char* b_tile;  // kSlices tiles, 1024-aligned
  int* ea;                // [64] row exponents of the two stacked op(A)
  int* eb;                // [64] column exponents of [op(B0) op(B1)]
  uint64_t* bar;          // [2] mbarriers: products reading A tile 0 / 1 done
  unsigned* mx;           // [128] high words of the row (0..63) / column (64..127) maxima; zero between calls
  uint32_t tmem;          // TMEM base address
  uint32_t uses[2];       // commits made on bar[0], bar[1] (uniform across the CTA)
  int m_last;             // block size of the last call (tiles hold zeros beyond it)
  int* abort;             // shared flag: a wait gave up
};

__device__ inline void small_zero_tiles(unsigned char* tiles) {
  uint4* z = reinterpret_cast<uint4*>(tiles);
  for (int i = threadIdx.x; i < (2 * kSmallATile + kSlices * kSmallBTile) / 16; i += blockDim.x)
    z[i] = make_uint4(0, 0, 0, 0);
}

// Byte offset of byte kbyte of row r in a swizzled tile.
__device__ __forceinline__ int sw_off(int r, int kbyte) {
  return r * 128 + ((((kbyte >> 4) ^ (r & 7)) & 7) << 4) + (kbyte & 15);
}

// Sets up the shared tiles (zeroed) and barriers; warp 0 allocates TMEM.
// Called by every thread of the CTA once, before the first product.
__device__ inline void small_init(SmallTC& t, unsigned char* smem_1024, int* abort_flag) {
  t.a_tile = smem_1024;
  t.b_tile = smem_1024 + 2 * kSmallATile;
  t.ea = reinterpret_cast<int*>(t.b_tile + kSlices * kSmallBTile);
  t.eb = t.ea + 64;
  t.bar = reinterpret_cast<uint64_t*>(t.eb + 64);
  t.mx = reinterpret_cast<unsigned*>(t.bar + 8);
  t.abort = abort_flag;
  for (int i = threadIdx.x; i < 128; i += blockDim.x) t.mx[i] = 0u;
  t.uses[0] = t.uses[1] = 0;
  t.m_last = 0;
  small_zero_tiles(smem_1024);
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(&t.bar[0]), 1);
    mbar_init(smem_u32(&t.bar[1]), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __shared__ uint32_t s_tmem;
  if ((threadIdx.x >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s_tmem)),
                 "r"(kSmallTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  t.tmem = s_tmem;
}

__device__ __forceinline__ void small_wait(SmallTC& t, int b);

// Frees TMEM once the last products have completed (bounded waits).
__device__ inline void small_release(SmallTC& t) {
  small_wait(t, 0);
  small_wait(t, 1);
  tc_fence_before();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(t.tmem), "r"(kSmallTmemCols));
}

// Bounded wait for the next completion on bar[b]; on time-out the CTA's
// abort flag is set (the products' results are then not used).
__device__ __forceinline__ void small_wait(SmallTC& t, int b) {
  if (t.uses[b] == 0) return;
  const bool ok = mbar_wait(smem_u32(&t.bar[b]), (t.uses[b] - 1) & 1);
  if (!ok) *t.abort = 1;
}

// F 2^s + lo 2^t as a double, rounded once, with two FP64 additions (the
// FP64 pipe is the narrow one on this part): F (|F| < 2^51) is scaled
// exactly by the magic-number form -- the bits of M = 1.5 2^(52+s) plus F
// are the double M + F 2^s, and subtracting M is exact -- and lo (FP32) is
// widened with its exponent moved by t through integer operations.  Out of
// the normal range (or lo subnormal) the plain conversions are used.
__device__ __forceinline__ double small_assemble(long long F, float lo, int s, int t) {
  const unsigned int lb = __float_as_uint(lo);
  const int le = (int)((lb >> 23) & 0xFF);
  const bool lo_zero = (lb & 0x7FFFFFFFu) == 0u;
  const int de = le - 127 + t + 1023;  // biased double exponent of lo 2^t
  if (s < -1070 || s > 960 || (!lo_zero && (le == 0 || de < 1 || de > 2046)))
    return scalbn((double)F, s) + scalbn((double)lo, t);
  const long long mb = ((long long)(1023 + 52 + s) << 52) | (1ll << 51);
  const double M = __longlong_as_double(mb);
  const double f = __longlong_as_double(mb + F) - M;
  const double l = lo_zero ? 0.0
                           : __longlong_as_double(((long long)(lb >> 31) << 63) | ((long long)de << 52) |
                                                  ((long long)(lb & 0x7FFFFFu) << 29));
  return f + l;
}

// C_kb = op(A_k) op(B_b) for k = 0, 1 and b < NB.  out(k, b, i, c, part,
// value) receives every real component (part 0 real, 1 imaginary) of
// element (i, c) of C_kb.  Returns false (results not written) when a wait
// gave up; every thread of the CTA (kSmallThreads) calls it.
template <int NB, class Out>
__device__ bool small_zgemm(SmallTC& t, int m, Op<double> A0, Op<double> A1, const Op<double> (&B)[NB],
                            const Out& out) {
  static_assert(NB >= 1 && NB <= kSmallNB, "right operands");
  if (blockDim.x != kSmallThreads) return false;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int mm = m * m;
  // (1) operands into registers; row maxima of op(A0), op(A1) and column
  // maxima of op(Bb) by atomics on the magnitudes' high words (enough for
  // the exponents; the words are zero on entry)
  cx<double> av[kSmallPerA], bv[NB][kSmallPerB];
#pragma unroll
  for (int u = 0; u < kSmallPerA; ++u) {
    const int idx = tid + u * kSmallThreads;
    av[u] = mk<double>(0.0, 0.0);
    if (idx < 2 * mm) {
      const int k = idx >= mm ? 1 : 0, e = idx - k * mm;
      const int i = e % m, j = e / m;
      av[u] = k == 0 ? A0.at(i, j) : A1.at(i, j);
      const unsigned long long x = mag_bits(av[u].x), y = mag_bits(av[u].y);
      atomicMax(&t.mx[k * 32 + i], (unsigned)((x > y ? x : y) >> 32));
    }
  }
#pragma unroll
  for (int b = 0; b < NB; ++b) {
#pragma unroll
    for (int u = 0; u < kSmallPerB; ++u) {
      const int idx = tid + u * kSmallThreads;
      bv[b][u] = mk<double>(0.0, 0.0);
      if (idx < mm) {
        const int j = idx % m, c = idx / m;
        bv[b][u] = B[b].at(j, c);
        const unsigned long long x = mag_bits(bv[b][u].x), y = mag_bits(bv[b][u].y);
        atomicMax(&t.mx[64 + b * 32 + c], (unsigned)((x > y ? x : y) >> 32));
      }
    }
  }
  // the previous call's MMAs may still read the tiles: wait for both buffers
  small_wait(t, 0);
  small_wait(t, 1);
  __syncthreads();
  if (m != t.m_last) {  // a smaller block leaves stale slices beyond it
    small_zero_tiles(t.a_tile);
    __syncthreads();
    t.m_last = m;
  }
  if (tid < 128) {
    const int e = exp_of_maxbits((unsigned long long)t.mx[tid] << 32);
    if (tid < 64)
      t.ea[tid] = e;
    else
      t.eb[tid - 64] = e;
  }
  // (2) all B slices: row 32 b + c of slice tile s holds [Re, Im] of
  // op(Bb)(j, c) at bf16 2j, 2j+1
#pragma unroll
  for (int b = 0; b < NB; ++b) {
#pragma unroll
    for (int u = 0; u < kSmallPerB; ++u) {
      const int idx = tid + u * kSmallThreads;
      if (idx < mm) {
        const int j = idx % m, c = idx / m;
        const int eb = exp_of_maxbits((unsigned long long)t.mx[64 + b * 32 + c] << 32);
        bool nre, nim;
        const unsigned long long Fr = fixed56(bv[b][u].x, eb, nre);
        const unsigned long long Fi = fixed56(bv[b][u].y, eb, nim);
        const int off = sw_off(b * 32 + c, 4 * j);
#pragma unroll
        for (int s = 1; s <= kSlices; ++s) {
          const uint32_t w = (uint32_t)slice_bf16(Fr, s, nre) | ((uint32_t)slice_bf16(Fi, s, nim) << 16);
          *reinterpret_cast<uint32_t*>(t.b_tile + (s - 1) * kSmallBTile + off) = w;
        }
      }
    }
  }
  // (3) fixed point of the A elements, kept for the eight slices
  unsigned long long Fr[kSmallPerA], Fi[kSmallPerA];
  unsigned negs = 0u;
  int aoff[kSmallPerA], aoff1[kSmallPerA];
#pragma unroll
  for (int u = 0; u < kSmallPerA; ++u) {
    const int idx = tid + u * kSmallThreads;
    Fr[u] = Fi[u] = 0ull;
    aoff[u] = aoff1[u] = -1;
    if (idx < 2 * mm) {
      const int k = idx >= mm ? 1 : 0, e = idx - k * mm;
      const int i = e % m, j = e / m;
      const int ea = exp_of_maxbits((unsigned long long)t.mx[k * 32 + i] << 32);
      bool nre, nim;
      Fr[u] = fixed56(av[u].x, ea, nre);
      Fi[u] = fixed56(av[u].y, ea, nim);
      negs |= (nre ? 1u : 0u) << (2 * u);
      negs |= (nim ? 2u : 0u) << (2 * u);
      aoff[u] = sw_off(k * 64 + 2 * i, 4 * j);
      aoff1[u] = sw_off(k * 64 + 2 * i + 1, 4 * j);
    }
  }
  constexpr uint32_t idesc = idesc_bf16(128, kSmallN * NB);
  unsigned inited = 0u;  // thread 0: slots written since the call began
  for (int s = 0; s < kSlices; ++s) {
    const int buf = s & 1;
    // the products of slice s-2 read this A tile (each thread waits itself)
    if (s >= 2) small_wait(t, buf);
    unsigned char* at = t.a_tile + buf * kSmallATile;
#pragma unroll
    for (int u = 0; u < kSmallPerA; ++u) {
      if (aoff[u] < 0) continue;
      const bool nre = (negs >> (2 * u)) & 1u, nim = (negs >> (2 * u)) & 2u;
      const uint16_t re = slice_bf16(Fr[u], s + 1, nre), im = slice_bf16(Fi[u], s + 1, nim);
      const uint16_t mim = im ? (uint16_t)(im ^ 0x8000u) : (uint16_t)0;
      // rows 2i and 2i+1 of the embedding: [Re, -Im] and [Im, Re]
      *reinterpret_cast<uint32_t*>(at + aoff[u]) = (uint32_t)re | ((uint32_t)mim << 16);
      *reinterpret_cast<uint32_t*>(at + aoff1[u]) = (uint32_t)im | ((uint32_t)re << 16);
    }
    // make the generic-proxy writes visible to the tensor cores
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    // every thread has read the maxima: clear them for the next call
    if (s == 0 && tid < 128) t.mx[tid] = 0u;
    if (tid == 0) {
      tc_fence_after();
      for (int tt = 0; s + tt <= kSlices - 1; ++tt) {
        const int slot = small_slot(s, tt);
        const uint32_t col = (uint32_t)(slot * kSmallSlotCols);
        const bool first = ((inited >> slot) & 1u) == 0u;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const uint64_t ad = desc_sw128(smem_u32(at + kk * 32));
          const uint64_t bd = desc_sw128(smem_u32(t.b_tile + tt * kSmallBTile + kk * 32));
          mma_bf16(t.tmem + col, ad, bd, idesc, (first && kk == 0) ? 0u : 1u);
        }
        inited |= 1u << slot;
      }
      mma_commit(smem_u32(&t.bar[buf]));
    }
    t.uses[buf] += 1;
  }
  small_wait(t, 0);
  small_wait(t, 1);
  __syncthreads();
  const bool ok = *t.abort == 0;
  if (ok) {
    tc_fence_after();
    // warp w reads TMEM lanes 32 (w & 3) .. +31 (rows of the tile) and
    // NB groups of 16 columns from column 16 NB (w >> 2)
    const int sub = warp & 3, half = warp >> 2;
    const int R = sub * 32 + lane;
    const int k = R >> 6, Rk = R & 63;
    const int i = Rk >> 1, part = Rk & 1;
    const int ea = t.ea[k * 32 + i];
#pragma unroll
    for (int g = 0; g < NB; ++g) {
      const int c0 = (half * NB + g) * 16;  // first column of the group
      const uint32_t base = t.tmem + ((uint32_t)(sub * 32) << 16) + (uint32_t)c0;
      uint32_t r[kSmallExact][16];
#pragma unroll
      for (int q = 0; q < kSmallExact; ++q) tmem_ld16_nowait(base + (uint32_t)(q * kSmallSlotCols), r[q]);
      tmem_wait_ld();
#pragma unroll
      for (int q = 0; q < kSmallExact; ++q) tmem_regs_ready(r[q]);
      long long F[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) F[j] = 0;
#pragma unroll
      for (int q = 0; q < kSmallExact; ++q) {
        const int d = q <= 3 ? q + 2 : kTopD;  // 1-based pair sum of the slot
        const float scale = __int_as_float((127 + kBeta * d) << 23);
        const int sh = kBeta * (kTopD - d);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const float f = fmaf(__uint_as_float(r[q][j]), scale, 12582912.0f);
          F[j] += (long long)(__float_as_int(f) - 0x4B400000) << sh;
        }
      }
      uint32_t lo[16];
      tmem_ld16(base + (uint32_t)(kSmallLow * kSmallSlotCols), lo);
      if (Rk < 2 * m) {
        const int b = c0 >> 5;  // right operand of this group
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int c = (c0 & 31) + j;
          if (c >= m) continue;
          const int eb = t.eb[b * 32 + c];
          double v;
          if (ea == kExpBad || eb == kExpBad) {
            v = __longlong_as_double(0x7FF8000000000000ll);
          } else {
            // F in units of 2^(ea + eb - 42), the light pairs in 2^(ea + eb)
            v = small_assemble(F[j], __uint_as_float(lo[j]), ea + eb - 42, ea + eb);
          }
          out(k, b, i, c, part, v);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  return ok;
}

// Epilogues of the decimation step (component-wise: part 0 real, 1
// imaginary); product (k, b) goes to c[k][b] by mode[k][b]
enum { OUT_STORE = 0, OUT_ACC = 1, OUT_ACC2 = 2 };
struct OutQuad {
  int mode[2][2];
  cx<double>* c[2][2];
  cx<double>* c2[2][2];  // second target of OUT_ACC2
  int ld;
  __device__ __forceinline__ void operator()(int k, int b, int i, int j, int part, double v) const {
    double* p = reinterpret_cast<double*>(c[k][b] + i + j * ld) + part;
    const int md = mode[k][b];
    if (md == OUT_STORE) {
      *p = v;
    } else {
      *p += v;
      if (md == OUT_ACC2) reinterpret_cast<double*>(c2[k][b] + i + j * ld)[part] += v;
    }
  }
};

}  // namespace tc
}  // namespace pf
