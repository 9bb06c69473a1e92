// CTA-level FP64-grade complex products of blocks up to 32 x 32 on tcgen05,
// for the lead decimations of the 32-wide mixed pipeline (the batched
// large products are in tc_abi.cu; the splitting is the same: every row of
// op(A) and column of op(B) scaled by a power of two and cut into eight
// 7-bit BF16 slices, slice pairs with s + t <= 6 summed exactly, the lighter
// ones in one FP32 accumulator, the result assembled in FP64).
//
// Layout: the CTA writes the slices itself into shared memory, in the
// K-major 128-byte-swizzled layout that the tcgen05 descriptors read (row r
// of a tile at r * 128 bytes, its 16-byte chunk c stored at chunk c ^ (r & 7)).
// A_big (2m x 2m, the interleaved real embedding of op(A)) occupies rows
// 0 .. 2m-1 of a 128-row tile (rows above stay zero: M = 128), B_big (m x 2m)
// rows 0 .. m-1 of a 32-row tile (N = 32); K = 2m <= 64 is one swizzle row.
// TMEM: 15 accumulators of 32 columns for the exact pairs and one for the
// light pairs (512 columns: the kernel runs one CTA per SM).  All 36 pair
// products of a GEMM are issued at once (B slices all resident, A slices
// double-buffered), then drained by the four warps that own TMEM lanes 0-63.
#pragma once
#include "cmat.cuh"
#include "tc_ptx.cuh"

namespace pf {
namespace tc {

constexpr int kSmallN = 32;                       // largest block
constexpr int kSmallATile = 128 * 128;            // bytes of one A slice tile
constexpr int kSmallBTile = kSmallN * 128;        // bytes of one B slice tile
constexpr int kSmallTmemCols = 512;
constexpr int kSmallLow = 15;                     // TMEM slot of the light pairs
constexpr int kSmallSmem = 2 * kSmallATile + kSlices * kSmallBTile + 3 * 32 * 4 + 64;

// slot of the exact pair (s, t) (0-based slices, s + t + 2 <= kTopD), in the
// order d = 2, 3, ..., kTopD; -1 for the light pairs
__device__ __forceinline__ int small_slot(int s, int t) {
  const int d = s + t;  // 0-based pair sum
  if (d + 2 > kTopD) return -1;
  return d * (d + 1) / 2 + s;
}
static_assert((kTopD - 1) * kTopD / 2 == kSmallLow, "15 exact pairs");

struct SmallTC {
  unsigned char* a_tile;  // 2 tiles, 1024-aligned
  unsigned char* b_tile;  // kSlices tiles, 1024-aligned
  int* ea;                // [64] row exponents of the two stacked op(A)
  int* eb;                // [32] column exponents of op(B)
  uint64_t* bar;          // [2] mbarriers: products reading A tile 0 / 1 done
  uint32_t tmem;          // TMEM base address
  uint32_t uses[2];       // commits made on bar[0], bar[1] (uniform across the CTA)
  int m_last;             // block size of the last product (tiles hold zeros beyond it)
  int* abort;             // shared flag: a wait gave up
};

__device__ inline void small_zero_tiles(unsigned char* tiles) {
  uint4* z = reinterpret_cast<uint4*>(tiles);
  for (int i = threadIdx.x; i < (2 * kSmallATile + kSlices * kSmallBTile) / 16; i += blockDim.x)
    z[i] = make_uint4(0, 0, 0, 0);
}

// Byte offset of element k (bf16 index) of row r in a swizzled tile.
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
  t.bar = reinterpret_cast<uint64_t*>(t.eb + 32);
  t.abort = abort_flag;
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

// Two products with a shared right operand in one M = 128 tile:
//   C0 = op(A0) op(B) (rows 0..2m-1 of the tile), C1 = op(A1) op(B) (rows
//   64..64+2m-1).  out(k, i, c, part, value) receives every real component
// of Ck.  Returns false (results not written) when a wait gave up; every
// thread of the CTA calls it (256 threads: the eight warps drain TMEM).
template <class Out>
__device__ bool small_zgemm2(SmallTC& t, int m, Op<double> A0, Op<double> A1, Op<double> B, const Out& out) {
  const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31;
  // exponents: rows of op(A0) (threads 0..m-1), op(A1) (32..), columns of op(B) (64..)
  if (tid < 96 && (tid & 31) < m) {
    const int k = tid >> 5, r = tid & 31;
    unsigned long long mx = 0;
    for (int j = 0; j < m; ++j) {
      const cx<double> a = k == 0 ? A0.at(r, j) : (k == 1 ? A1.at(r, j) : B.at(j, r));
      const unsigned long long x = mag_bits(a.x), y = mag_bits(a.y);
      mx = x > mx ? x : mx;
      mx = y > mx ? y : mx;
    }
    if (k < 2)
      t.ea[k * 32 + r] = exp_of_maxbits(mx);
    else
      t.eb[r] = exp_of_maxbits(mx);
  }
  // the previous product's MMAs may still read the tiles: wait for both buffers
  small_wait(t, 0);
  small_wait(t, 1);
  __syncthreads();
  if (m != t.m_last) {  // a smaller block leaves stale slices beyond it
    small_zero_tiles(t.a_tile);
    __syncthreads();
    t.m_last = m;
  }
  // all B slices: row c of tile s holds [Re, Im] of op(B)(j, c) at bf16 2j, 2j+1
  for (int idx = tid; idx < m * m; idx += nt) {
    const int j = idx % m, c = idx / m;
    cx<double> b = B.at(j, c);
    bool nre, nim;
    const unsigned long long Fr = fixed56(b.x, t.eb[c], nre);
    const unsigned long long Fi = fixed56(b.y, t.eb[c], nim);
#pragma unroll
    for (int s = 1; s <= kSlices; ++s) {
      const uint32_t w = (uint32_t)slice_bf16(Fr, s, nre) | ((uint32_t)slice_bf16(Fi, s, nim) << 16);
      *reinterpret_cast<uint32_t*>(t.b_tile + (s - 1) * kSmallBTile + sw_off(c, 4 * j)) = w;
    }
  }
  constexpr uint32_t idesc = idesc_bf16(128, kSmallN);
  bool low_init = false;
  for (int s = 0; s < kSlices; ++s) {
    const int buf = s & 1;
    // the products of slice s-2 read this A tile
    if (s >= 2) small_wait(t, buf);
    __syncthreads();
    unsigned char* at = t.a_tile + buf * kSmallATile;
    for (int idx = tid; idx < 2 * m * m; idx += nt) {
      const int k = idx / (m * m), e = idx % (m * m);
      const int i = e % m, j = e / m;
      const cx<double> a = k == 0 ? A0.at(i, j) : A1.at(i, j);
      const int ev = t.ea[k * 32 + i];
      bool nre, nim;
      const unsigned long long Fr = fixed56(a.x, ev, nre);
      const unsigned long long Fi = fixed56(a.y, ev, nim);
      const uint16_t re = slice_bf16(Fr, s + 1, nre), im = slice_bf16(Fi, s + 1, nim);
      const uint16_t mim = im ? (uint16_t)(im ^ 0x8000u) : (uint16_t)0;
      const int row = k * 64 + 2 * i;
      *reinterpret_cast<uint32_t*>(at + sw_off(row, 4 * j)) = (uint32_t)re | ((uint32_t)mim << 16);
      *reinterpret_cast<uint32_t*>(at + sw_off(row + 1, 4 * j)) = (uint32_t)im | ((uint32_t)re << 16);
    }
    // make the generic-proxy writes visible to the tensor cores
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      for (int tt = 0; s + tt <= kSlices - 1; ++tt) {
        const int slot = small_slot(s, tt);
        const uint32_t col = (uint32_t)((slot >= 0 ? slot : kSmallLow) * kSmallN);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const uint64_t ad = desc_sw128(smem_u32(at + kk * 32));
          const uint64_t bd = desc_sw128(smem_u32(t.b_tile + tt * kSmallBTile + kk * 32));
          const uint32_t acc = slot >= 0 ? (uint32_t)(kk != 0) : (uint32_t)(low_init || kk != 0);
          mma_bf16(t.tmem + col, ad, bd, idesc, acc);
        }
        if (slot < 0) low_init = true;
      }
      mma_commit(smem_u32(&t.bar[buf]));
    }
    t.uses[buf] += 1;
  }
  small_wait(t, 0);
  small_wait(t, 1);
  __syncthreads();
  const bool ok = *t.abort == 0;
  if (ok && nt >= 256) {
    tc_fence_after();
    // warp w reads TMEM lanes 32 (w & 3) .. +31 (rows of the tile) and the
    // column half w >> 2
    const int sub = warp & 3, half = warp >> 2;
    if (half < 2) {
      const int R = sub * 32 + lane;
      const uint32_t base = t.tmem + ((uint32_t)(sub * 32) << 16) + (uint32_t)(half * 16);
      long long F[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) F[j] = 0;
      for (int d = 2; d <= kTopD; ++d) {
        const float scale = __int_as_float((127 + kBeta * d) << 23);
        const int sh = kBeta * (kTopD - d);
        for (int s = 0; s <= d - 2; ++s) {
          uint32_t r[16];
          tmem_ld16(base + (uint32_t)(small_slot(s, d - 2 - s) * kSmallN), r);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const float f = fmaf(__uint_as_float(r[j]), scale, 12582912.0f);
            F[j] += (long long)(__float_as_int(f) - 0x4B400000) << sh;
          }
        }
      }
      uint32_t r[16];
      tmem_ld16(base + (uint32_t)(kSmallLow * kSmallN), r);
      const int k = R >> 6, Rk = R & 63;
      const int i = Rk >> 1, part = Rk & 1;
      if (Rk < 2 * m) {
        const int ea = t.ea[k * 32 + i];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int c = half * 16 + j;
          if (c >= m) continue;
          const int eb = t.eb[c];
          double v;
          if (ea == kExpBad || eb == kExpBad)
            v = __longlong_as_double(0x7FF8000000000000ll);
          else
            v = scalbn((double)F[j] * 0x1p-42 + (double)__uint_as_float(r[j]), ea + eb);
          out(k, i, c, part, v);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  return ok;
}

// Epilogues of the decimation step (component-wise: part 0 real, 1
// imaginary; k selects the stacked product)
enum { OUT_STORE = 0, OUT_ACC = 1, OUT_ACC2 = 2 };
struct OutPair {
  int mode[2];
  cx<double>* c[2];
  cx<double>* c2[2];  // second target of OUT_ACC2
  int ld;
  __device__ __forceinline__ void operator()(int k, int i, int j, int part, double v) const {
    double* p = reinterpret_cast<double*>(c[k] + i + j * ld) + part;
    if (mode[k] == OUT_STORE) {
      *p = v;
    } else {
      *p += v;
      if (mode[k] == OUT_ACC2) reinterpret_cast<double*>(c2[k] + i + j * ld)[part] += v;
    }
  }
};

}  // namespace tc
}  // namespace pf
