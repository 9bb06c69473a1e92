// Warp-per-point layer engine for cross-sections up to 32 (n, nl, nr <= 32).
//
// After the lead decimations (one CTA per point, double-float) the layer
// recursion of the mixed path -- FP32 block LU of the extended matrix, FP32
// back substitution of the last block column, double-float residual
// refinement and the double-float Caroli trace -- runs with ONE WARP PER
// POINT and no CTA barriers:
//   * lane r holds row r of the left operand of a product in registers (32
//     complex floats), loaded from global memory (coalesced across lanes) or
//     from the warp's shared memory;
//   * the right operand lives in one of the warp's two shared 32 x 32
//     buffers and is read by broadcast; results go back to shared memory
//     (and to the per-point slabs) column by column;
//   * the block inverse is an in-shared-memory Gauss-Jordan with implicit
//     partial pivoting (no row exchanges; the final permutation is applied
//     when the factor is stored: inv(A)[k, P[j]] = M[P[k], j]).
// Every matrix is padded to 32 x 32: padded rows/columns of the couplings are
// zero and padded diagonal entries of the inverted blocks are one, so the
// padding never mixes into the physical part.
#pragma once
#include "mixed.cuh"

namespace pf {
namespace wp {

constexpr int NW = 32;   // padded block size
constexpr int LDW = 34;  // shared leading dimension: 16-byte aligned columns

// Per-point lead data written by the leads kernel (column-major, ld = 32).
struct LeadOut {
  fcx* g0;     // [npts][32*32] FP32 gl_ret = g_adv^H (left factor g_0)
  fcx* fsr;    // [npts][32*32] FP32 Sigma_R
  dcx* esl;    // [npts][32*32] df64 es_adv^H (A_00 = zL - esl)
  dcx* sr;     // [npts][32*32] df64 Sigma_R
  dcx* gml;    // [npts][32*32] df64 Gamma_L (wrapper sign)
  dcx* gmr;    // [npts][32*32] df64 Gamma_R
};

// Per-point slabs of the layer engine (column-major, ld = 32).
struct Slabs {
  fcx* lu;   // [pts][L+2][32*32] FP32 factors
  fcx* yv;   // [pts][L+2][32*32] FP32 forward vectors
  dcx* xv;   // [pts][L+2][32*32] df64 solution blocks
  float* corr; // [pts] size of the last sweep's correction of X_0 relative to X_0
};

__device__ __forceinline__ fcx fz() { return mk<float>(0.f, 0.f); }
__device__ __forceinline__ fcx ffma(fcx a, fcx b, fcx c) { return cfma(a, b, c); }

// Products are row-stationary: lane r holds row r of the left operand in
// registers (32 complex floats), the right operand sits in the warp's shared
// memory and is read by broadcast, and the result goes to an epilogue
// functor element by element (lane r, column c).  The column loop is not
// unrolled, so one product is a few hundred instructions of code: the
// layer loops stay resident in the instruction cache (a fully unrolled
// 32 x 32 x 32 product is ~75 KB of code per call site).

// a[k] = S(lane, k) of a shared-memory block (ld LDW)
__device__ __forceinline__ void row_smem(const fcx* S, int lane, fcx (&a)[NW]) {
#pragma unroll
  for (int k = 0; k < NW; ++k) a[k] = S[lane + k * LDW];
}
// a[k] = conj(S(k, lane)): row `lane` of S^H
__device__ __forceinline__ void row_smem_h(const fcx* S, int lane, fcx (&a)[NW]) {
  const float4* col = reinterpret_cast<const float4*>(S + lane * LDW);
#pragma unroll
  for (int k2 = 0; k2 < NW / 2; ++k2) {
    const float4 v = col[k2];
    a[2 * k2] = mk<float>(v.x, -v.y);
    a[2 * k2 + 1] = mk<float>(v.z, -v.w);
  }
}
// a[k] = M(lane, k) of a padded global block (ld NW)
__device__ __forceinline__ void row_block(const fcx* M, int lane, fcx (&a)[NW]) {
#pragma unroll
  for (int k = 0; k < NW; ++k) a[k] = M[lane + k * NW];
}

// For c = 0..31: epi(lane, c, sum_k a[k] B(k, c)), B in shared memory (ld LDW).
template <class Epi>
__device__ __forceinline__ void rgemm(const fcx (&a)[NW], const fcx* B, int lane, Epi epi) {
  constexpr int U = 4;  // columns per step: 8 independent FMA chains per lane
#pragma unroll 1
  for (int c0 = 0; c0 < NW; c0 += U) {
    fcx acc0[U], acc1[U];
#pragma unroll
    for (int u = 0; u < U; ++u) acc0[u] = acc1[u] = fz();
#pragma unroll
    for (int k = 0; k < NW; k += 2) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const float4 b = *reinterpret_cast<const float4*>(B + k + (c0 + u) * LDW);
        acc0[u] = ffma(a[k], mk<float>(b.x, b.y), acc0[u]);
        acc1[u] = ffma(a[k + 1], mk<float>(b.z, b.w), acc1[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) epi(lane, c0 + u, cadd(acc0[u], acc1[u]));
  }
}

// rgemm over the NC columns [cb, cb + NC) of B only (NC a multiple of 4).
template <int NC, class Epi>
__device__ __forceinline__ void rgemm_cols(const fcx (&a)[NW], const fcx* B, int lane, int cb, Epi epi) {
  constexpr int U = 4;
#pragma unroll 1
  for (int c0 = cb; c0 < cb + NC; c0 += U) {
    fcx acc0[U], acc1[U];
#pragma unroll
    for (int u = 0; u < U; ++u) acc0[u] = acc1[u] = fz();
#pragma unroll
    for (int k = 0; k < NW; k += 2) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const float4 b = *reinterpret_cast<const float4*>(B + k + (c0 + u) * LDW);
        acc0[u] = ffma(a[k], mk<float>(b.x, b.y), acc0[u]);
        acc1[u] = ffma(a[k + 1], mk<float>(b.z, b.w), acc1[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) epi(lane, c0 + u, cadd(acc0[u], acc1[u]));
  }
}

// Operand V_j (dims dj x d(j+1)) of the extended system as a global view.
struct GView {
  const fcx* p;
  int ldg, rows, cols;
  bool ct;
};
__device__ __forceinline__ GView vview(const MSys& s, int q, int j) {
  const int n = s.n, L = s.L;
  GView g;
  if (j == 0) {
    g.p = s.fHld + (size_t)q * s.nl * n;
    g.ldg = s.nl;
    g.rows = s.nl;
    g.cols = n;
    g.ct = false;
  } else if (j == L) {
    g.p = s.fHrd + (size_t)q * s.nr * n;  // V_L = Hrd^H (n x nr)
    g.ldg = s.nr;
    g.rows = n;
    g.cols = s.nr;
    g.ct = true;
  } else {
    g.p = s.fHdv + ((size_t)q * (L - 1) + (j - 1)) * n * n;
    g.ldg = n;
    g.rows = n;
    g.cols = n;
    g.ct = false;
  }
  return g;
}
__device__ __forceinline__ GView vview_h(const MSys& s, int q, int j) {
  GView g = vview(s, q, j);
  const int t = g.rows;
  g.rows = g.cols;
  g.cols = t;
  g.ct = !g.ct;
  return g;
}
// Element (r, k) of a view (zero outside rows x cols).
__device__ __forceinline__ fcx view_at(const GView& g, int r, int k) {
  if (r >= g.rows || k >= g.cols) return fz();
  return g.ct ? cconj(g.p[k + (size_t)r * g.ldg]) : g.p[r + (size_t)k * g.ldg];
}
// a[k] = g(lane, k)
__device__ __forceinline__ void row_view(const GView& g, int lane, fcx (&a)[NW]) {
#pragma unroll
  for (int k = 0; k < NW; ++k) a[k] = view_at(g, lane, k);
}
// Stage a view into the warp's smem buffer (lane r writes row r).
__device__ __forceinline__ void stage_rows(fcx* S, const GView& g, int lane) {
#pragma unroll
  for (int k = 0; k < NW; ++k) S[lane + k * LDW] = view_at(g, lane, k);
}

// In-place Gauss-Jordan inverse of the 32x32 matrix in S with implicit
// partial pivoting (pivot = first max |re|+|im| among unused rows), then
// the unscrambled inverse is written to D (smem) and optionally to global
// (ld 32).  Lane r owns row r, so every shared access is either a row-r
// element (consecutive lanes, conflict free) or a broadcast of the pivot
// row.  Returns status bits (uniform).
__device__ inline int winverse(fcx* S, fcx* D, fcx* gout, int lane) {
  unsigned used = 0u;
  int status = PF_OK;
  int perm_mine = 0;  // P[lane]: pivot row of step `lane`
  int step_mine = 0;  // the step whose pivot row was `lane`
  for (int k = 0; k < NW; ++k) {
    const fcx mk_ = S[lane + k * LDW];
    float v = fabsf(mk_.x) + fabsf(mk_.y);
    if (v != v) v = 3.0e38f;
    if (used & (1u << lane)) v = -1.f;
    int bi = lane;
    float bv = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > bv || (ov == bv && oi < bi)) {
        bv = ov;
        bi = oi;
      }
    }
    const int p = bi;
    if (lane == k) perm_mine = p;
    if (lane == p) step_mine = k;
    const fcx piv = mk<float>(__shfl_sync(0xffffffffu, mk_.x, p), __shfl_sync(0xffffffffu, mk_.y, p));
    if (piv.x == 0.f && piv.y == 0.f) status |= PF_SINGULAR;
    if (!(isfinite(piv.x) && isfinite(piv.y))) status |= PF_NAN;
    const fcx ip = crecip(piv);
    fcx rowp[NW];
#pragma unroll
    for (int c = 0; c < NW; ++c) rowp[c] = S[p + c * LDW];
    __syncwarp();
    // row r != p becomes row_r - m_r row_p with m_r = S(r, k) / piv, and
    // column k becomes -m; the pivot row becomes row_p / piv, i.e. the same
    // update from a zero row with m = -1/piv (column k: 1/piv)
    const bool prow = lane == p;
    const fcx m = prow ? mk<float>(-ip.x, -ip.y) : cmul(mk_, ip);
#pragma unroll
    for (int c = 0; c < NW; ++c) {
      const fcx old = prow ? fz() : S[lane + c * LDW];
      const fcx nv = mk<float>(old.x - (m.x * rowp[c].x - m.y * rowp[c].y),
                               old.y - (m.x * rowp[c].y + m.y * rowp[c].x));
      S[lane + c * LDW] = (c == k) ? mk<float>(-m.x, -m.y) : nv;
    }
    used |= 1u << p;
    __syncwarp();
  }
  // inv[k, P[j]] = M[P[k], j]: lane r = P[k] moves its row to row k
#pragma unroll
  for (int j = 0; j < NW; ++j) {
    const int pj = __shfl_sync(0xffffffffu, perm_mine, j);
    const fcx e = S[lane + j * LDW];
    D[step_mine + pj * LDW] = e;
    if (gout) gout[step_mine + pj * NW] = e;
  }
  __syncwarp();
  return status;
}

// Extended-layer dimension
__device__ __forceinline__ int edim(const MSys& s, int j) { return j == 0 ? s.nl : (j == s.L + 1 ? s.nr : s.n); }

// df64 zero
__device__ __forceinline__ dcx dz() { return mk<df64>(df64(0.f, 0.f), df64(0.f, 0.f)); }

}  // namespace wp
}  // namespace pf
