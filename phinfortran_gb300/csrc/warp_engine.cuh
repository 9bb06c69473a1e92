// Warp-per-point layer engine for cross-sections up to 32 (n, nl, nr <= 32).
//
// After the lead decimations (one CTA per point, double-float) the layer
// recursion of the mixed path -- FP32 block LU of the extended matrix, FP32
// back substitution of the last block column, double-float residual
// refinement and the double-float Caroli trace -- runs with ONE WARP PER
// POINT and no CTA barriers:
//   * lane c owns column c of the right-hand operand and of the result, in
//     registers (32 complex floats);
//   * the left operand of every product lives in the warp's own shared
//     memory and is read by broadcast (all lanes read the same element);
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
};

__device__ __forceinline__ fcx fz() { return mk<float>(0.f, 0.f); }
__device__ __forceinline__ fcx ffma(fcx a, fcx b, fcx c) { return cfma(a, b, c); }

// c[:] = A(smem, ld LDW) * b[:]   (lane's column)
__device__ __forceinline__ void wgemm(const fcx* A, const fcx (&b)[NW], fcx (&c)[NW]) {
#pragma unroll
  for (int r = 0; r < NW; ++r) c[r] = fz();
#pragma unroll
  for (int k = 0; k < NW; ++k) {
    const fcx bk = b[k];
    const float4* col = reinterpret_cast<const float4*>(A + k * LDW);
#pragma unroll
    for (int r2 = 0; r2 < NW / 2; ++r2) {
      const float4 a = col[r2];
      c[2 * r2] = ffma(mk<float>(a.x, a.y), bk, c[2 * r2]);
      c[2 * r2 + 1] = ffma(mk<float>(a.z, a.w), bk, c[2 * r2 + 1]);
    }
  }
}
// c[:] = A^H * b[:]   (A in smem; row k of A read as column k of A^H)
__device__ __forceinline__ void wgemm_ct(const fcx* A, const fcx (&b)[NW], fcx (&c)[NW]) {
#pragma unroll
  for (int r = 0; r < NW; ++r) c[r] = fz();
#pragma unroll
  for (int k = 0; k < NW; ++k) {
    const fcx bk = b[k];
#pragma unroll
    for (int r = 0; r < NW; ++r) c[r] = ffma(cconj(A[k + r * LDW]), bk, c[r]);
  }
}

// Lane c loads column c of an (rows x cols) column-major global block with
// leading dimension ldg (zero padding), optionally conjugate-transposed.
__device__ __forceinline__ void load_col(const fcx* M, int ldg, int rows, int cols, bool ct, int c, fcx (&v)[NW]) {
#pragma unroll
  for (int r = 0; r < NW; ++r) {
    fcx e = fz();
    if (!ct) {
      if (r < rows && c < cols) e = M[r + (size_t)c * ldg];
    } else {
      // element (r, c) of M^H = conj(M(c, r)); M is cols x rows here
      if (r < rows && c < cols) e = cconj(M[c + (size_t)r * ldg]);
    }
    v[r] = e;
  }
}
__device__ __forceinline__ void store_col_smem(fcx* S, int c, const fcx (&v)[NW]) {
#pragma unroll
  for (int r = 0; r < NW; ++r) S[r + c * LDW] = v[r];
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
// Stage V_j into the warp's smem buffer (lane c writes column c).
__device__ __forceinline__ void stage_v(fcx* S, const GView& g, int c) {
  fcx v[NW];
  load_col(g.p, g.ldg, g.rows, g.cols, g.ct, c, v);
  store_col_smem(S, c, v);
  __syncwarp();
}

// In-place Gauss-Jordan inverse of the 32x32 matrix in S with implicit
// partial pivoting (pivot = first max |re|+|im| among unused rows), then
// the unscrambled inverse is written to D (smem) and optionally to global
// (ld 32).  Returns status bits (uniform).
__device__ int winverse(fcx* S, fcx* D, fcx* gout, int lane) {
  unsigned used = 0u;
  int status = PF_OK;
  int perm_mine = 0;  // P[lane]
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
    const fcx piv = S[p + k * LDW];
    if (piv.x == 0.f && piv.y == 0.f) status |= PF_SINGULAR;
    if (!(isfinite(piv.x) && isfinite(piv.y))) status |= PF_NAN;
    const fcx ip = crecip(piv);
    fcx colk[NW];
#pragma unroll
    for (int r = 0; r < NW; ++r) colk[r] = S[r + k * LDW];
    const fcx rowp = S[p + lane * LDW];
    __syncwarp();
    if (lane == k) {
#pragma unroll
      for (int r = 0; r < NW; ++r) {
        const fcx t = cmul(colk[r], ip);
        S[r + k * LDW] = (r == p) ? ip : mk<float>(-t.x, -t.y);
      }
    } else {
      const fcx f = cmul(rowp, ip);
#pragma unroll
      for (int r = 0; r < NW; ++r) {
        const fcx old = S[r + lane * LDW];
        const fcx nv = mk<float>(old.x - (colk[r].x * f.x - colk[r].y * f.y),
                                 old.y - (colk[r].x * f.y + colk[r].y * f.x));
        S[r + lane * LDW] = (r == p) ? f : nv;
      }
    }
    used |= 1u << p;
    __syncwarp();
  }
  // inv[k, P[c]] = M[P[k], c]: lane c moves its column to column P[c]
  const int pc = perm_mine;  // lane c holds P[c]
#pragma unroll
  for (int k = 0; k < NW; ++k) {
    const int pk = __shfl_sync(0xffffffffu, perm_mine, k);
    const fcx e = S[pk + lane * LDW];
    D[k + pc * LDW] = e;
    if (gout) gout[k + pc * NW] = e;
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
