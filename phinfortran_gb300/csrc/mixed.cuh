// Mixed-precision point pipeline (FP32 + double-float, no FP64 instructions
// on the hot path).
//
// The transmission T_L = Re Tr[G_{0,N+1} Gamma_R G_{0,N+1}^H Gamma_L] of
// negf/lesser.f90:787-792 only needs the last block column
// X = A^{-1} E_{N+1} of the extended block-tridiagonal matrix A over the
// layers j = 0 (left lead cell), 1..L (device), L+1 (right lead cell):
//   A_00      = gl^{-1} = conj(z_adv) - es_adv^H   (es: decimated onsite)
//   A_jj      = z_D - Hd_j                        (j = 1..L)
//   A_{L+1}   = z_D - HR - Sigma_R                (lesser.f90:617)
//   A_{j,j+1} = -V_j  with V_0 = Hld, V_j = Hdv_j, V_L = Hrd^H.
// The reference's left-connected recursion (lesser.f90:547-654) is the
// forward block-LU of this matrix, so G_{0,N+1} = X_0.
//
// Stages per point:
//   1. both lead decimations in df64 (the FP64 algorithm of
//      negf/surface.f90:488-497; FP32 cannot resolve eta ~ 1e-6);
//   2. FP32 block LU: g_j = inv(A_jj - V_{j-1}^H g_{j-1} V_{j-1}), stored;
//   3. FP32 back substitution X_{L+1} = g_{L+1}, X_j = g_j V_j X_{j+1};
//   4. `nref` refinement sweeps: residual r = E_{N+1} - A X in df64,
//      correction by the stored FP32 factors, X += dX in df64;
//   5. Caroli trace in df64.
#pragma once
#include "tc_small.cuh"
#include "transport.cuh"

namespace pf {

using dcx = cx<df64>;
using fcx = cx<float>;

// Block set converted once per call: df64 copies (residual, leads, Caroli)
// and FP32 copies (factorisation and corrections), same layout as the
// FP64 input (column-major, ld = rows).
// Row-compressed (ELL) copy of a block family: row r of block b keeps up to
// K (column, value) pairs at [(b*K + k)*rows + r] (slot-major, so the rows a
// warp reads at one slot are contiguous); column -1 ends the row.
struct Ell {
  const int* col;
  const dcx* val;
  int K, rows;
};
__host__ __device__ __forceinline__ size_t ell_at(size_t blk, int K, int rows, int r, int k) {
  return (blk * K + k) * (size_t)rows + r;
}

enum { PF_ELL_K = 16 };

// Adaptive refinement: a sweep after the first runs only for the points
// whose previous correction of X_0 (the block the Caroli trace reads) was
// above PF_REFINE_TOL relative to X_0 (largest entry against largest
// entry).  On the disordered 32-wide tight-binding ribbon (L = 200, 1024
// energies, eta 1e-6) about a quarter of the points are above 3e-5 after
// the first sweep, and they include every point whose T was still more
// than 1e-8 away from a reproducible FP64 result.
constexpr float PF_REFINE_TOL = 3.0e-5f;

struct MSys {
  int n, nl, nr, L, nq;
  const dcx *HL, *HLv, *HR, *HRv, *Hd, *Hdv, *Hld, *Hrd;
  const fcx *fHR, *fHd, *fHdv, *fHld, *fHrd;
  // sparse copies for the residual: Hd, Hdv, Hdv^H, Hld, Hld^H, Hrd, Hrd^H;
  // used when *ell_overflow == 0 (every row of every block has <= K nonzeros)
  Ell eHd, eHdv, eHdvH, eHld, eHldH, eHrd, eHrdH;
  const int* ell_overflow;
  // FP64 lead blocks (the caller's arrays) and the lead arithmetic:
  // PF_LEAD_FP64 whole decimations in FP64, PF_LEAD_DF64 in double-float,
  // PF_LEAD_SPLIT the first PF_LEAD_FP64_STEPS steps in FP64, the rest in
  // double-float
  const cx<double> *dHL, *dHLv, *dHR, *dHRv;
  int lead_mode;
};
enum { PF_LEAD_FP64 = 0, PF_LEAD_DF64 = 1, PF_LEAD_SPLIT = 2 };

// Lopez-Sancho steps carried in FP64 before the split decimation continues in
// double-float.  On the disordered 32-wide ribbon (1024 energies, eta 1e-6)
// the split decimation halves the number of energies whose T misses FP64 by
// more than 1e-8 (53 instead of 114; 2 instead of 6 among the FP64-
// reproducible ones); only whole FP64 decimations remove them all, so the
// split is an option for speed, not the default.
constexpr int PF_LEAD_FP64_STEPS = 8;

enum { NSM_M = 6 };
// per-CTA df64 scratch matrices
enum { M_E1 = 0, M_ES, M_W2, M_W3, M_ESL, M_GML, M_GMR, M_SR, M_R, NGM };

struct MCtx {
  dcx* sm[NSM_M];      // shared slots, sized for df64 (reused as FP32)
  dcx* gs[NGM];        // per-CTA df64 scratch
  fcx* lu;             // (L+2) FP32 factors g_j
  fcx* yv;             // (L+2) FP32 forward vectors
  dcx* xv;             // (L+2) df64 solution blocks X_j
  fcx* fsr;            // FP32 copy of Sigma_R
  int ld;
  size_t mat;          // elements per matrix slot
  InvWork<df64> iwd;
  InvWork<float> iwf;
  double* red;
};

__device__ __forceinline__ fcx f_of(dcx a) { return mk<float>(a.x.hi, a.y.hi); }
__device__ __forceinline__ dcx d_of(fcx a) { return mk<df64>(df64(a.x, 0.f), df64(a.y, 0.f)); }

// dst(float) = src(df64) or its conjugate transpose
__device__ inline void cvt_df_to_f(fcx* dst, int ldd, bool conj_t, const dcx* src, int lds, int m, int n) {
  for (int i = threadIdx.x; i < m * n; i += blockDim.x) {
    const int r = i % m, c = i / m;
    const dcx v = conj_t ? cconj(src[c + r * lds]) : src[r + c * lds];
    dst[r + (size_t)c * ldd] = f_of(v);
  }
  __syncthreads();
}
__device__ inline void cvt_f_to_df(dcx* dst, int ldd, const fcx* src, int lds, int m, int n) {
  for (int i = threadIdx.x; i < m * n; i += blockDim.x) {
    const int r = i % m, c = i / m;
    dst[r + (size_t)c * ldd] = d_of(src[r + c * lds]);
  }
  __syncthreads();
}

// Epilogue: C(float) = acc + add(r,c)   (add from a float matrix, optional)
struct EpiStoreAddF {
  fcx* c;
  int ld;
  const fcx* add;
  int ldadd;
  __device__ __forceinline__ void operator()(int r, int col, fcx acc) const {
    fcx v = acc;
    if (add) v = cadd(v, add[r + col * ldadd]);
    c[r + col * ld] = v;
  }
};
// Epilogue of the backward correction: d = acc + y (float); stores d and
// accumulates X += d in df64.
struct EpiCorr {
  fcx* d;
  int ld;
  const fcx* y;
  dcx* x;
  __device__ __forceinline__ void operator()(int r, int col, fcx acc) const {
    const fcx v = cadd(acc, y[r + col * ld]);
    d[r + col * ld] = v;
    dcx xv = x[r + col * ld];
    xv.x = xv.x + df64(v.x, 0.f);
    xv.y = xv.y + df64(v.y, 0.f);
    x[r + col * ld] = xv;
  }
};
// Residual start: R = acc + b - z X   (b = I on the last layer)
struct EpiRes0 {
  dcx* r;
  int ld;
  const dcx* X;
  dcx z;
  bool ident;
  __device__ __forceinline__ void operator()(int i, int col, dcx acc) const {
    const dcx xv = X[i + col * ld];
    dcx v = csub(acc, cmul(z, xv));
    if (ident && i == col) v.x = v.x + df64(1.f, 0.f);
    r[i + col * ld] = v;
  }
};

// dst (type A) = src (type B) or its conjugate transpose, through FP64
template <typename A, typename B>
__device__ void copy_cvt(cx<A>* dst, int ldd, bool conj_t, const cx<B>* src, int lds, int m, int n) {
  for (int i = threadIdx.x; i < m * n; i += blockDim.x) {
    const int r = i % m, c = i / m;
    const cx<B> v = conj_t ? cconj(src[c + r * lds]) : src[r + c * lds];
    cx<A> o;
    o.x = conv<A>(to_d(v.x));
    o.y = conv<A>(to_d(v.y));
    dst[r + (size_t)c * ldd] = o;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Lead decimations in FP64 (the algorithm and arithmetic of the plain FP64
// path, negf/surface.f90:488-497), results converted to the layouts of the
// df64 variant below.  The decimation is the part of the mixed pipeline
// that double-float cannot carry at eta ~ 1e-6: with 48-bit decimations 114
// of the disordered ribbon's 1024 energies end more than 1e-8 from FP64 (6
// of them FP64-reproducible, up to 4.4e-8), with FP64 decimations every
// energy is within 2.2e-9.  The doubling iteration amplifies its rounding
// errors (a relative error of alpha or beta doubles with every step), and a
// residual of the surface function does not single the bad energies out
// (FP64 decimations leave residuals up to 2e-7 there too), so every point
// takes FP64 decimations.  The CTA's df64-sized slots hold the FP64
// matrices (both 16 bytes per complex element).
// ---------------------------------------------------------------------------
// The FP64 decimation (negf/surface.f90:479-497) with its six block
// products per step on the tensor cores (FP64-grade slice products, see
// tc_small.cuh) and the inverse in FP64 on the CTA.  On return SM2 holds
// g = inv(z - es) and G_ES holds es (FP64), as after decimate<double>.
// FP64 Gauss-Jordan inverse of an n x n block (n <= 32) for the
// tensor-core decimation, by a CTA of 256 threads, with look-ahead.  The
// matrix alternates between M and T (step k reads one and writes the other,
// so nothing is read after it is overwritten) and a step needs one barrier:
// warp 0 writes column k+1 of step k's result, picks the pivot of step k+1
// (first maximum of |re| + |im| among the unused rows, as inverse()) and
// forms its reciprocal and the multipliers f(r) = a(r, k+1) / pivot, while
// warps 1-7 write the other columns.  Elimination in multiplier form:
// a'(r, c) = a(r, c) - f(r) a(p, c), a'(p, c) = a(p, c) / pivot,
// a'(r, k) = -f(r), a'(p, k) = 1 / pivot.  The row and column order is
// restored by one gather, inv(k, P(j)) = A(P(k), j).  fbuf holds two
// buffers of m multipliers (the pivot row's entry carries 1 / pivot); the
// status bits (PF_SINGULAR, PF_NAN) are those of inverse().
// Helpers of the tensor-core decimation that keep work off the FP64 pipe.
// W = z - e: the negation as a flip of the sign bit (integer operation),
// one FP64 addition on the diagonal.
__device__ inline void shift_neg_bits(cx<double>* dst, int ldd, cx<double> z, const cx<double>* src, int lds, int n) {
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
    const int r = i % n, c = i / n;
    const cx<double> v = src[r + c * lds];
    cx<double> w = mk<double>(__longlong_as_double(__double_as_longlong(v.x) ^ (long long)0x8000000000000000ull),
                              __longlong_as_double(__double_as_longlong(v.y) ^ (long long)0x8000000000000000ull));
    if (r == c) w = mk<double>(z.x - v.x, z.y - v.y);
    dst[r + c * ldd] = w;
  }
  __syncthreads();
}

// max_ij |a_ij| for the stopping test, as the square root of the largest
// re^2 + im^2 (two FP64 operations an entry instead of hypot's scaled
// evaluation; equal to a few ulps, so the stopping step can differ from the
// FP64 path's only when the test value sits within rounding of the
// threshold).  NaN propagates.
__device__ inline double max_mod_sq(const cx<double>* a, int ld, int m, double* red) {
  double v = 0.0;
  for (int i = threadIdx.x; i < m * m; i += blockDim.x) {
    const cx<double> e = a[i % m + (i / m) * ld];
    const double h = fma(e.x, e.x, e.y * e.y);
    v = (h > v || h != h) ? h : v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w > v || w != w) ? w : v;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      const double w = __shfl_xor_sync(0xffffffffu, v, o);
      v = (w > v || w != w) ? w : v;
    }
    if (lane == 0) red[0] = sqrt(v);
  }
  __syncthreads();
  v = red[0];
  __syncthreads();
  return v;
}

struct LaWork {
  cx<double>* f;  // [2 m]
  int* perm;      // [n]
  int* flag;      // [1]
  int m;
};

__device__ __forceinline__ cx<double> la_recip(cx<double> a) {
  // 1 / a = conj(a) / |a|^2 with a scaled by s = 2^-e, 2^e <= max(|re|, |im|)
  // < 2^(e+1), so that |a s|^2 neither overflows nor underflows
  const double mx = fmax(fabs(a.x), fabs(a.y));
  if (!(mx > 0.0) || !(mx <= 1.7976931348623157e308)) {
    const double nan = __longlong_as_double(0x7FF8000000000000ll);
    return mk<double>(nan, nan);
  }
  const int e = ilogb(mx);
  if (e < -1020 || e > 1020) return crecip(a);  // scale factor out of range: Smith's form
  const double sc = scalbn(1.0, -e);
  const double sx = a.x * sc, sy = a.y * sc;
  const double r = 1.0 / fma(sx, sx, sy * sy);
  return mk<double>(sx * r * sc, -sy * r * sc);
}

// Warp 0: pivot of the column v (lane r holds row r) among the unused rows;
// writes the multipliers, 1 / pivot at the pivot's slot and perm[k].
__device__ __forceinline__ int la_pivot(cx<double> v, int lane, int n, bool used, cx<double>* f, int* perm_k) {
  const double a = cabs1(v);
  double best = (lane < n && !used) ? ((a != a) ? 3.0e300 : a) : -1.0;
  int bi = (lane < n && !used) ? lane : 64;
  for (int o = 16; o > 0; o >>= 1) {
    const double ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ob > best || (ob == best && oi < bi)) {
      best = ob;
      bi = oi;
    }
  }
  const int p = bi < n ? bi : 0;
  const cx<double> piv = mk<double>(__shfl_sync(0xffffffffu, v.x, p), __shfl_sync(0xffffffffu, v.y, p));
  int st = PF_OK;
  if (piv.x == 0.0 && piv.y == 0.0) st |= PF_SINGULAR;
  if (!(isfinite(piv.x) && isfinite(piv.y))) st |= PF_NAN;
  const cx<double> ip = la_recip(piv);
  if (lane < n) f[lane] = lane == p ? ip : cmul(v, ip);
  if (lane == 0) *perm_k = p;
  return st;
}

__device__ inline int inverse_la(cx<double>* M, cx<double>* T, int ld, int n, LaWork w) {
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  int st = PF_OK;
  bool used = false;  // warp 0, lane r: row r has been a pivot
  if (warp == 0) st |= la_pivot(lane < n ? M[lane] : mk<double>(0.0, 0.0), lane, n, false, w.f, w.perm);
  __syncthreads();
  cx<double>* src = M;
  cx<double>* dst = T;
  for (int k = 0; k < n; ++k) {
    const cx<double>* f = w.f + (k & 1) * w.m;
    const int p = w.perm[k];
    const cx<double> ip = f[p];
    if (warp == 0) {
      if (k + 1 < n) {
        cx<double> v = mk<double>(0.0, 0.0);
        if (lane < n) {
          const cx<double> ap = src[p + (k + 1) * ld];
          if (lane == p) {
            v = cmul(ap, ip);
          } else {
            const cx<double> fr = f[lane];
            v = src[lane + (k + 1) * ld];
            v.x = fma(-fr.x, ap.x, fma(fr.y, ap.y, v.x));
            v.y = fma(-fr.x, ap.y, fma(-fr.y, ap.x, v.y));
          }
          dst[lane + (k + 1) * ld] = v;
        }
        if (lane == p) used = true;
        st |= la_pivot(v, lane, n, used, w.f + ((k + 1) & 1) * w.m, w.perm + k + 1);
      }
    } else {
      for (int i = tid - 32; i < n * n; i += nt - 32) {
        const int r = i % n, c = i / n;
        if (c == k + 1) continue;
        cx<double> o;
        if (c == k) {
          o = r == p ? ip : mk<double>(-f[r].x, -f[r].y);
        } else if (r == p) {
          o = cmul(src[p + c * ld], ip);
        } else {
          const cx<double> fr = f[r], a = src[p + c * ld];
          o = src[r + c * ld];
          o.x = fma(-fr.x, a.x, fma(fr.y, a.y, o.x));
          o.y = fma(-fr.x, a.y, fma(-fr.y, a.x, o.y));
        }
        dst[r + c * ld] = o;
      }
    }
    __syncthreads();
    cx<double>* t = src;
    src = dst;
    dst = t;
  }
  // src holds the permuted inverse
  for (int i = tid; i < n * n; i += nt) {
    const int r = i % n, c = i / n;
    dst[r + w.perm[c] * ld] = src[w.perm[r] + c * ld];
  }
  if (tid == 0) *w.flag = st;
  __syncthreads();
  if (dst != M) {
    for (int i = tid; i < n * n; i += nt) {
      const int r = i % n, c = i / n;
      M[r + c * ld] = dst[r + c * ld];
    }
  }
  st = *w.flag;
  __syncthreads();
  return st;
}

template <int S>
__device__ int decimate_tc(const Ctx<double>& c, tc::SmallTC& t, int m, cx<double> z, Op<double> h00,
                           Op<double> a0, Op<double> b0, double conv, int max_iter, int* iters_out) {
  const int ld = c.ld;
  cx<double>* al = c.sm[0];
  cx<double>* be = c.sm[1];
  cx<double>* W1 = c.sm[2];
  cx<double>* e1 = c.gs[G_E1];
  cx<double>* es = c.gs[G_ES];
  cx<double>* W2 = c.gs[G_W2];
  cx<double>* W3 = c.gs[G_W3];
  int st = PF_OK;
  // look-ahead inverse: the multipliers in the inverse workspace (rowk and
  // colk are contiguous, 2 m entries), the second matrix buffer in SM3
  const LaWork la{c.iw.rowk, c.iw.perm, c.iw.flag, m};
  copy_in(e1, ld, h00, m, m);
  copy_in(es, ld, h00, m, m);
  copy_in(al, ld, a0, m, m);
  copy_in(be, ld, b0, m, m);
  double maxdiff = max_mod_sq(al, ld, m, c.red);
  int it = 0;
  while (maxdiff > conv) {
    if (it >= max_iter) {
      st |= PF_NOT_CONVERGED;
      break;
    }
    shift_neg_bits(W1, ld, z, e1, ld, m);                                                 // z - e1
    st |= inverse_la(W1, c.sm[3], ld, m, la);                                        // ive
    // the six products of a step as two tensor-core calls:
    //   [W2; W3] = [alpha; beta] ive, then
    //   [W2; W3] [beta alpha] = [W2 beta, W2 alpha; W3 beta, W3 alpha]:
    //   e1, es += W2 beta; alpha' = W2 alpha; beta' = W3 beta; e1 += W3 alpha
    // (the last through W3, whose values are in registers by then, so that
    // e1 receives its two sums in the order of the FP64 step)
    using tc::OutQuad;
    const Op<double> b1[1] = {opN<double>(W1, ld)};
    bool ok = tc::small_zgemm<1>(t, m, opN<double>(al, ld), opN<double>(be, ld), b1,
                                 OutQuad{{{tc::OUT_STORE, 0}, {tc::OUT_STORE, 0}},
                                         {{W2, nullptr}, {W3, nullptr}},
                                         {{nullptr, nullptr}, {nullptr, nullptr}},
                                         ld});
    const Op<double> b2[2] = {opN<double>(be, ld), opN<double>(al, ld)};
    ok = ok && tc::small_zgemm<2>(t, m, opN<double>(W2, ld), opN<double>(W3, ld), b2,
                                  OutQuad{{{tc::OUT_ACC2, tc::OUT_STORE}, {tc::OUT_STORE, tc::OUT_STORE}},
                                          {{e1, al}, {be, W3}},
                                          {{es, nullptr}, {nullptr, nullptr}},
                                          ld});
    if (!ok) {
      st |= PF_TC_TIMEOUT;
      break;
    }
    for (int i = threadIdx.x; i < m * m; i += blockDim.x) {
      const int r = i % m, cc = i / m;
      const cx<double> w = W3[r + cc * ld];
      cx<double>& e = e1[r + cc * ld];
      e.x += w.x;
      e.y += w.y;
    }
    __syncthreads();
    maxdiff = max_mod_sq(al, ld, m, c.red);
    ++it;
  }
  if (maxdiff != maxdiff) st |= PF_NAN;
  shift_neg_bits(W1, ld, z, es, ld, m);
  st |= inverse_la(W1, c.sm[3], ld, m, la);
  if (iters_out) *iters_out = it;
  return st;
}

template <int S>
__device__ int mixed_leads64(const MCtx& mc, const MSys& sys, int q, double E, const Params& P, int* it_l,
                             int* it_r, tc::SmallTC* tcx = nullptr) {
  Ctx<double> c;
  for (int i = 0; i < NSM; ++i) c.sm[i] = reinterpret_cast<cx<double>*>(mc.sm[i]);
  c.gs[G_E1] = reinterpret_cast<cx<double>*>(mc.gs[M_E1]);
  c.gs[G_ES] = reinterpret_cast<cx<double>*>(mc.gs[M_ES]);
  c.gs[G_W2] = reinterpret_cast<cx<double>*>(mc.gs[M_W2]);
  c.gs[G_W3] = reinterpret_cast<cx<double>*>(mc.gs[M_W3]);
  c.ld = mc.ld;
  c.iw.rowk = reinterpret_cast<cx<double>*>(mc.iwd.rowk);
  c.iw.colk = reinterpret_cast<cx<double>*>(mc.iwd.colk);
  c.iw.perm = mc.iwd.perm;
  c.iw.flag = mc.iwd.flag;
  c.red = mc.red;
  const int ld = mc.ld, nl = sys.nl, nr = sys.nr;
  const double eps = E * P.eta + P.eta0;
  int st = PF_OK;
  cx<double>* tmp = reinterpret_cast<cx<double>*>(mc.gs[M_W2]);
  {
    const cx<double>* HL = sys.dHL + (size_t)q * nl * nl;
    const cx<double>* HLv = sys.dHLv + (size_t)q * nl * nl;
    if (tcx)
      st |= decimate_tc<S>(c, *tcx, nl, mk<double>(E, -eps), opN<double>(HL, nl), opC<double>(HLv, nl),
                           opN<double>(HLv, nl), P.convergence, P.max_iter, it_l);
    else
      st |= decimate<double, S>(c, nl, mk<double>(E, -eps), opN<double>(HL, nl), opC<double>(HLv, nl),
                                opN<double>(HLv, nl), P.convergence, P.max_iter, it_l);
    copy_cvt<float, double>(mc.lu, ld, true, c.sm[2], ld, nl, nl);             // g_0 = g_adv^H
    copy_cvt<df64, double>(mc.gs[M_ESL], ld, true, c.gs[G_ES], ld, nl, nl);    // es_adv^H
    lead_sigma<double, S>(c, nl, HLv);                                         // SM1 = sl_adv
    gamma_from_sigma(tmp, ld, c.sm[1], ld, nl, -1);
    copy_cvt<df64, double>(mc.gs[M_GML], ld, false, tmp, ld, nl, nl);
  }
  if (P.lead_mirror && P.lead_mirror[q]) {
    copy_cvt<df64, double>(mc.gs[M_SR], ld, true, c.sm[1], ld, nl, nl);
    copy_cvt<float, double>(mc.fsr, ld, true, c.sm[1], ld, nl, nl);
    copy_out(mc.gs[M_GMR], ld, false, mc.gs[M_GML], ld, nl, nl);
    if (it_r) *it_r = *it_l;
  } else {
    const cx<double>* HR = sys.dHR + (size_t)q * nr * nr;
    const cx<double>* HRv = sys.dHRv + (size_t)q * nr * nr;
    if (tcx)
      st |= decimate_tc<S>(c, *tcx, nr, mk<double>(E, eps), opN<double>(HR, nr), opC<double>(HRv, nr),
                           opN<double>(HRv, nr), P.convergence, P.max_iter, it_r);
    else
      st |= decimate<double, S>(c, nr, mk<double>(E, eps), opN<double>(HR, nr), opC<double>(HRv, nr),
                                opN<double>(HRv, nr), P.convergence, P.max_iter, it_r);
    lead_sigma<double, S>(c, nr, HRv);                                         // SM1 = sr_ret
    copy_cvt<df64, double>(mc.gs[M_SR], ld, false, c.sm[1], ld, nr, nr);
    copy_cvt<float, double>(mc.fsr, ld, false, c.sm[1], ld, nr, nr);
    gamma_from_sigma(tmp, ld, c.sm[1], ld, nr, +1);
    copy_cvt<df64, double>(mc.gs[M_GMR], ld, false, tmp, ld, nr, nr);
  }
  return st;
}

// One Lopez-Sancho step (negf/surface.f90:488-497) on the state in c:
// alpha = SM0, beta = SM1, e1 = G_E1, es = G_ES; SM2, G_W2, G_W3 scratch.
template <typename R, int S>
__device__ int sancho_step(const Ctx<R>& c, int m, cx<R> z) {
  const int ld = c.ld;
  cx<R>* al = c.sm[0];
  cx<R>* be = c.sm[1];
  cx<R>* W1 = c.sm[2];
  cx<R>* e1 = c.gs[G_E1];
  cx<R>* es = c.gs[G_ES];
  cx<R>* W2 = c.gs[G_W2];
  cx<R>* W3 = c.gs[G_W3];
  shift_neg(W1, ld, z, e1, ld, m);                                                              // z - e1
  const int st = inverse(W1, ld, m, c.iw);                                                      // ive
  row_gemm<R, S>(m, m, m, opN<R>(al, ld), opN<R>(W1, ld), EpiStore<R>{W2, ld, mk<R>(1, 0)});  // alpha ive
  row_gemm<R, S>(m, m, m, opN<R>(be, ld), opN<R>(W1, ld), EpiStore<R>{W3, ld, mk<R>(1, 0)});  // beta ive
  row_gemm<R, S>(m, m, m, opN<R>(W2, ld), opN<R>(be, ld), EpiAcc2<R>{e1, es, ld});
  row_gemm<R, S>(m, m, m, opN<R>(W3, ld), opN<R>(al, ld), EpiAcc<R>{e1, ld});
  row_gemm<R, S>(m, m, m, opN<R>(W2, ld), opN<R>(al, ld), EpiStore<R>{W2, ld, mk<R>(1, 0)});
  row_gemm<R, S>(m, m, m, opN<R>(W3, ld), opN<R>(be, ld), EpiStore<R>{W3, ld, mk<R>(1, 0)});
  copy_in(al, ld, opN<R>(W2, ld), m, m);
  copy_in(be, ld, opN<R>(W3, ld), m, m);
  return st;
}

// In-place FP64 -> df64 of an m x m slot (both 16 bytes per complex element;
// every element is read and written by the same thread).
__device__ inline void slot_to_df64(dcx* a, int ld, int m) {
  for (int i = threadIdx.x; i < m * m; i += blockDim.x) {
    const int r = i % m, c = i / m;
    const cx<double> v = reinterpret_cast<const cx<double>*>(a)[r + c * ld];
    a[r + c * ld] = mk<df64>(df64(v.x), df64(v.y));
  }
  __syncthreads();
}

// Split decimation: the FP64 algorithm of negf/surface.f90:479-497 with the
// first PF_LEAD_FP64_STEPS steps in FP64 and the rest in df64 (the state is
// converted in place).  On return SM2 holds g = inv(z - es) and G_ES holds
// es, both df64, as after decimate<df64>.
template <int S>
__device__ int decimate_split(const Ctx<df64>& cd, int m, double E, double eps_signed, const cx<double>* h00,
                              const cx<double>* v, double conv, int max_iter, int* iters_out) {
  Ctx<double> c;
  for (int i = 0; i < NSM; ++i) c.sm[i] = reinterpret_cast<cx<double>*>(cd.sm[i]);
  for (int i : {(int)G_E1, (int)G_ES, (int)G_W2, (int)G_W3}) c.gs[i] = reinterpret_cast<cx<double>*>(cd.gs[i]);
  c.ld = cd.ld;
  c.iw.rowk = reinterpret_cast<cx<double>*>(cd.iw.rowk);
  c.iw.colk = reinterpret_cast<cx<double>*>(cd.iw.colk);
  c.iw.perm = cd.iw.perm;
  c.iw.flag = cd.iw.flag;
  c.red = cd.red;
  const int ld = cd.ld;
  copy_in(c.gs[G_E1], ld, opN<double>(h00, m), m, m);
  copy_in(c.gs[G_ES], ld, opN<double>(h00, m), m, m);
  copy_in(c.sm[0], ld, opC<double>(v, m), m, m);  // alpha0 = V^H
  copy_in(c.sm[1], ld, opN<double>(v, m), m, m);  // beta0 = V
  int st = PF_OK;
  double maxdiff = max_abs(c.sm[0], ld, m, m, c.red);
  int it = 0;
  const cx<double> z64 = mk<double>(E, eps_signed);
  while (maxdiff > conv && it < PF_LEAD_FP64_STEPS && it < max_iter) {
    st |= sancho_step<double, S>(c, m, z64);
    maxdiff = max_abs(c.sm[0], ld, m, m, c.red);
    ++it;
  }
  slot_to_df64(cd.sm[0], ld, m);
  slot_to_df64(cd.sm[1], ld, m);
  slot_to_df64(cd.gs[G_E1], ld, m);
  slot_to_df64(cd.gs[G_ES], ld, m);
  const dcx z = mk<df64>(df64(E), df64(eps_signed));
  while (maxdiff > conv) {
    if (it >= max_iter) {
      st |= PF_NOT_CONVERGED;
      break;
    }
    st |= sancho_step<df64, S>(cd, m, z);
    maxdiff = max_abs(cd.sm[0], ld, m, m, cd.red);
    ++it;
  }
  if (maxdiff != maxdiff) st |= PF_NAN;
  shift_neg(cd.sm[2], ld, z, cd.gs[G_ES], ld, m);
  st |= inverse(cd.sm[2], ld, m, cd.iw);
  if (iters_out) *iters_out = it;
  return st;
}

// ---------------------------------------------------------------------------
// Lead decimations in df64 (whole or split; FP64 when sys.lead_mode is
// PF_LEAD_FP64).  Results left in per-CTA scratch:
//   M_ESL = es_adv^H (df64), M_GML = -gml_adv, M_GMR = gmr_ret, M_SR = sr_ret,
//   lu[0] = gl_ret = g_adv^H (FP32), fsr = FP32 sr_ret.
// ---------------------------------------------------------------------------
template <int S>
__device__ int mixed_leads(const MCtx& mc, const MSys& sys, int q, double E, const Params& P, int* it_l,
                           int* it_r, tc::SmallTC* tcx = nullptr) {
  if (sys.lead_mode == PF_LEAD_FP64) return mixed_leads64<S>(mc, sys, q, E, P, it_l, it_r, tcx);
  const bool split = sys.lead_mode == PF_LEAD_SPLIT;
  Ctx<df64> c;
  for (int i = 0; i < NSM; ++i) c.sm[i] = mc.sm[i];
  c.gs[G_E1] = mc.gs[M_E1];
  c.gs[G_ES] = mc.gs[M_ES];
  c.gs[G_W2] = mc.gs[M_W2];
  c.gs[G_W3] = mc.gs[M_W3];
  c.ld = mc.ld;
  c.iw = mc.iwd;
  c.red = mc.red;
  const int ld = mc.ld, nl = sys.nl, nr = sys.nr;
  const double eps = E * P.eta + P.eta0;
  int st = PF_OK;
  {
    const dcx* HL = sys.HL + (size_t)q * nl * nl;
    const dcx* HLv = sys.HLv + (size_t)q * nl * nl;
    if (split)
      st |= decimate_split<S>(c, nl, E, -eps, sys.dHL + (size_t)q * nl * nl, sys.dHLv + (size_t)q * nl * nl,
                              P.convergence, P.max_iter, it_l);
    else
      st |= decimate<df64, S>(c, nl, mk<df64>(df64(E), df64(-eps)), opN<df64>(HL, nl), opC<df64>(HLv, nl),
                              opN<df64>(HLv, nl), P.convergence, P.max_iter, it_l);
    cvt_df_to_f(mc.lu, ld, true, c.sm[2], ld, nl, nl);          // g_0 = g_adv^H
    copy_out(mc.gs[M_ESL], ld, true, c.gs[G_ES], ld, nl, nl);   // es_adv^H
    lead_sigma<df64, S>(c, nl, HLv);                            // SM1 = sl_adv
    gamma_from_sigma(mc.gs[M_GML], ld, c.sm[1], ld, nl, -1);
  }
  if (P.lead_mirror && P.lead_mirror[q]) {
    // identical leads: sr_ret = sl_adv^H, gmr_ret = -gml_adv (see lead_pair)
    copy_out(mc.gs[M_SR], ld, true, c.sm[1], ld, nl, nl);
    cvt_df_to_f(mc.fsr, ld, true, c.sm[1], ld, nl, nl);
    copy_out(mc.gs[M_GMR], ld, false, mc.gs[M_GML], ld, nl, nl);
    if (it_r) *it_r = *it_l;
  } else {
    const dcx* HR = sys.HR + (size_t)q * nr * nr;
    const dcx* HRv = sys.HRv + (size_t)q * nr * nr;
    if (split)
      st |= decimate_split<S>(c, nr, E, eps, sys.dHR + (size_t)q * nr * nr, sys.dHRv + (size_t)q * nr * nr,
                              P.convergence, P.max_iter, it_r);
    else
      st |= decimate<df64, S>(c, nr, mk<df64>(df64(E), df64(eps)), opN<df64>(HR, nr), opC<df64>(HRv, nr),
                              opN<df64>(HRv, nr), P.convergence, P.max_iter, it_r);
    lead_sigma<df64, S>(c, nr, HRv);                            // SM1 = sr_ret
    copy_out(mc.gs[M_SR], ld, false, c.sm[1], ld, nr, nr);
    cvt_df_to_f(mc.fsr, ld, false, c.sm[1], ld, nr, nr);
    gamma_from_sigma(mc.gs[M_GMR], ld, c.sm[1], ld, nr, +1);
  }
  return st;
}

// Dimension of extended layer j.
__device__ __forceinline__ int ext_dim(const MSys& s, int j) { return j == 0 ? s.nl : (j == s.L + 1 ? s.nr : s.n); }

// Coupling V_j = -A_{j,j+1} (rows dim(j), cols dim(j+1)) as an FP32 operand.
__device__ __forceinline__ Op<float> vf(const MSys& s, int q, int j) {
  const int n = s.n, L = s.L;
  if (j == 0) return opN<float>(s.fHld + (size_t)q * s.nl * n, s.nl);
  if (j == L) return opC<float>(s.fHrd + (size_t)q * s.nr * n, s.nr);
  return opN<float>(s.fHdv + ((size_t)q * (L - 1) + (j - 1)) * n * n, n);
}
__device__ __forceinline__ Op<float> vf_h(const MSys& s, int q, int j) {
  Op<float> o = vf(s, q, j);
  o.ct = !o.ct;
  return o;
}
__device__ __forceinline__ Op<df64> vd(const MSys& s, int q, int j) {
  const int n = s.n, L = s.L;
  if (j == 0) return opN<df64>(s.Hld + (size_t)q * s.nl * n, s.nl);
  if (j == L) return opC<df64>(s.Hrd + (size_t)q * s.nr * n, s.nr);
  return opN<df64>(s.Hdv + ((size_t)q * (L - 1) + (j - 1)) * n * n, n);
}
__device__ __forceinline__ Op<df64> vd_h(const MSys& s, int q, int j) {
  Op<df64> o = vd(s, q, j);
  o.ct = !o.ct;
  return o;
}

// ---------------------------------------------------------------------------
// Stage 2+3: FP32 block LU of the extended system and back substitution.
// ---------------------------------------------------------------------------
template <int S>
__device__ int mixed_factor_solve(const MCtx& mc, const MSys& sys, int q, fcx zD) {
  const int ld = mc.ld, L = sys.L;
  const size_t mat = mc.mat;
  fcx* sV = reinterpret_cast<fcx*>(mc.sm[0]);
  fcx* sT = reinterpret_cast<fcx*>(mc.sm[1]);
  fcx* sA = reinterpret_cast<fcx*>(mc.sm[2]);
  fcx* sX = reinterpret_cast<fcx*>(mc.sm[3]);
  int st = PF_OK;
  Op<float> none = opN<float>(nullptr, 1);
  for (int j = 1; j <= L + 1; ++j) {
    const int dp = ext_dim(sys, j - 1), dj = ext_dim(sys, j);
    const Op<float> V = vf(sys, q, j - 1);               // dp x dj
    copy_in(sV, ld, V, dp, dj);                            // stage V (B operand)
    row_gemm<float, S>(dp, dj, dp, opN<float>(mc.lu + (j - 1) * mat, ld), opN<float>(sV, ld),
                       EpiStore<float>{sT, ld, mk<float>(1.f, 0.f)});      // T = g_{j-1} V
    EpiShift<float> epi;
    epi.c = sA;
    epi.ld = ld;
    epi.z = zD;
    if (j <= L) {
      epi.h = opN<float>(sys.fHd + ((size_t)q * L + (j - 1)) * sys.n * sys.n, sys.n);
      epi.has_h = true;
      epi.s = none;
      epi.has_s = false;
    } else {
      epi.h = opN<float>(sys.fHR + (size_t)q * sys.nr * sys.nr, sys.nr);
      epi.has_h = true;
      epi.s = opN<float>(mc.fsr, ld);
      epi.has_s = true;
    }
    row_gemm<float, S>(dj, dj, dp, opC<float>(sV, ld), opN<float>(sT, ld), epi);  // A_j - V^H T
    st |= inverse(sA, ld, dj, mc.iwf);
    copy_out(mc.lu + j * mat, ld, false, sA, ld, dj, dj);
  }
  // back substitution for the last block column
  const int nr = sys.nr;
  copy_out(sX, ld, false, mc.lu + (L + 1) * mat, ld, nr, nr);   // X_{L+1} = g_{L+1}
  cvt_f_to_df(mc.xv + (L + 1) * mat, ld, sX, ld, nr, nr);
  for (int j = L; j >= 0; --j) {
    const int dj = ext_dim(sys, j), dn = ext_dim(sys, j + 1);
    const Op<float> V = vf(sys, q, j);                   // dj x dn
    row_gemm<float, S>(dj, nr, dn, V, opN<float>(sX, ld), EpiStore<float>{sT, ld, mk<float>(1.f, 0.f)});
    row_gemm<float, S>(dj, nr, dj, opN<float>(mc.lu + j * mat, ld), opN<float>(sT, ld),
                       EpiStore<float>{sX, ld, mk<float>(1.f, 0.f)});
    cvt_f_to_df(mc.xv + j * mat, ld, sX, ld, dj, nr);
  }
  return st;
}

// Accumulate acc += M(r,:) X(:,c) over the ELL row of M.
__device__ __forceinline__ dcx ell_row_dot(const Ell& e, size_t blk, int r, const dcx* X, int ld, int c, dcx acc) {
  for (int k = 0; k < e.K; ++k) {
    const size_t at = ell_at(blk, e.K, e.rows, r, k);
    const int cc = e.col[at];
    if (cc < 0) break;
    acc = cfma(e.val[at], X[cc + c * ld], acc);
  }
  return acc;
}

// Interior residual layer j (1..L) with sparse blocks, one pass:
// R = - z X_j + Hd_j X_j + V_{j-1}^H X_{j-1} + V_j X_{j+1}
__device__ inline void residual_sparse(const MSys& s, int q, int j, dcx zD, const dcx* Xm, const dcx* X0, const dcx* Xp,
                                dcx* R, int ld) {
  const int n = s.n, nr = s.nr, L = s.L;
  for (int i = threadIdx.x; i < n * nr; i += blockDim.x) {
    const int r = i / nr, c = i % nr;   // consecutive threads share the row: broadcast ELL loads
    dcx acc = csub(czero<df64>(), cmul(zD, X0[r + c * ld]));
    acc = ell_row_dot(s.eHd, (size_t)q * L + (j - 1), r, X0, ld, c, acc);
    if (j == 1)
      acc = ell_row_dot(s.eHldH, (size_t)q, r, Xm, ld, c, acc);
    else
      acc = ell_row_dot(s.eHdvH, (size_t)q * (L - 1) + (j - 2), r, Xm, ld, c, acc);
    if (j == L)
      acc = ell_row_dot(s.eHrdH, (size_t)q, r, Xp, ld, c, acc);
    else
      acc = ell_row_dot(s.eHdv, (size_t)q * (L - 1) + (j - 1), r, Xp, ld, c, acc);
    R[r + c * ld] = acc;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Stage 4: one refinement sweep (df64 residual, FP32 correction).
// ---------------------------------------------------------------------------
// true when the correction of X_0 (d, rows < nl, columns < nr) is above
// PF_REFINE_TOL relative to X_0; the same answer on every thread of the CTA
__device__ inline bool refine_again(const fcx* d, const dcx* x, int ld, int nl, int nr, double* red) {
  float md = 0.f, mx = 0.f;
  for (int i = threadIdx.x; i < nl * nr; i += blockDim.x) {
    const int r = i % nl, c = i / nl;
    const fcx v = d[r + c * ld];
    const dcx u = x[r + c * ld];
    md = fmaxf(md, fabsf(v.x) + fabsf(v.y));
    mx = fmaxf(mx, fabsf(u.x.hi) + fabsf(u.y.hi));
  }
  for (int o = 16; o > 0; o >>= 1) {
    md = fmaxf(md, __shfl_xor_sync(0xffffffffu, md, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  float2* r2 = reinterpret_cast<float2*>(red);  // 32 doubles hold 32 pairs
  __syncthreads();
  if ((threadIdx.x & 31) == 0) r2[threadIdx.x >> 5] = make_float2(md, mx);
  __syncthreads();
  float a = 0.f, b = 0.f;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
    a = fmaxf(a, r2[w].x);
    b = fmaxf(b, r2[w].y);
  }
  __syncthreads();
  return a > PF_REFINE_TOL * b;
}

// One refinement sweep; returns whether another sweep would still change
// X_0 by more than PF_REFINE_TOL.
template <int S>
__device__ bool mixed_refine(const MCtx& mc, const MSys& sys, int q, dcx zL, dcx zD) {
  const int ld = mc.ld, L = sys.L, nr = sys.nr;
  const size_t mat = mc.mat;
  // df64 window of X blocks (B operands) and FP32 work slots
  dcx* xw[3] = {mc.sm[0], mc.sm[1], mc.sm[2]};
  fcx* sR = reinterpret_cast<fcx*>(mc.sm[3]);
  fcx* sYp = reinterpret_cast<fcx*>(mc.sm[4]);
  fcx* sY = reinterpret_cast<fcx*>(mc.sm[5]);
  dcx* R = mc.gs[M_R];
  const bool sparse = sys.ell_overflow != nullptr && *sys.ell_overflow == 0;
  // window: xw[0] = X_{j-1}, xw[1] = X_j, xw[2] = X_{j+1}
  copy_in(xw[1], ld, opN<df64>(mc.xv, ld), ext_dim(sys, 0), nr);
  for (int j = 0; j <= L + 1; ++j) {
    const int dj = ext_dim(sys, j);
    if (j + 1 <= L + 1) copy_in(xw[2], ld, opN<df64>(mc.xv + (j + 1) * mat, ld), ext_dim(sys, j + 1), nr);
    // r_j = b_j - z X_j + Hpart X_j + V_{j-1}^H X_{j-1} + V_j X_{j+1}
    if (j >= 1 && j <= L && sparse) {
      residual_sparse(sys, q, j, zD, xw[0], xw[1], xw[2], R, ld);
    } else {
      if (j == 0) {
        row_gemm<df64, S>(dj, nr, dj, opN<df64>(mc.gs[M_ESL], ld), opN<df64>(xw[1], ld),
                          EpiRes0{R, ld, xw[1], zL, false});
      } else if (j <= L) {
        row_gemm<df64, S>(dj, nr, dj, opN<df64>(sys.Hd + ((size_t)q * L + (j - 1)) * sys.n * sys.n, sys.n),
                          opN<df64>(xw[1], ld), EpiRes0{R, ld, xw[1], zD, false});
      } else {
        row_gemm<df64, S>(dj, nr, dj, opN<df64>(sys.HR + (size_t)q * nr * nr, nr), opN<df64>(xw[1], ld),
                          EpiRes0{R, ld, xw[1], zD, true});
        row_gemm<df64, S>(dj, nr, dj, opN<df64>(mc.gs[M_SR], ld), opN<df64>(xw[1], ld), EpiAcc<df64>{R, ld});
      }
      if (j >= 1)
        row_gemm<df64, S>(dj, nr, ext_dim(sys, j - 1), vd_h(sys, q, j - 1), opN<df64>(xw[0], ld),
                          EpiAcc<df64>{R, ld});
      if (j <= L)
        row_gemm<df64, S>(dj, nr, ext_dim(sys, j + 1), vd(sys, q, j), opN<df64>(xw[2], ld), EpiAcc<df64>{R, ld});
    }
    cvt_df_to_f(sR, ld, false, R, ld, dj, nr);
    // forward: y_j = g_j (r_j + V_{j-1}^H y_{j-1})
    if (j >= 1)
      row_gemm<float, S>(dj, nr, ext_dim(sys, j - 1), vf_h(sys, q, j - 1), opN<float>(sYp, ld),
                         EpiStoreAddF{sR, ld, sR, ld});
    row_gemm<float, S>(dj, nr, dj, opN<float>(mc.lu + j * mat, ld), opN<float>(sR, ld),
                       EpiStoreAddF{sY, ld, nullptr, 0});
    copy_out(mc.yv + j * mat, ld, false, sY, ld, dj, nr);
    fcx* t = sYp;
    sYp = sY;
    sY = t;
    dcx* u = xw[0];
    xw[0] = xw[1];
    xw[1] = xw[2];
    xw[2] = u;
  }
  // backward: d_{L+1} = y_{L+1}; d_j = y_j + g_j V_j d_{j+1}; X += d
  fcx* sD = sYp;   // holds y_{L+1}
  fcx* sT = sR;
  fcx* sN = sY;
  {
    dcx* x = mc.xv + (L + 1) * mat;
    for (int i = threadIdx.x; i < nr * nr; i += blockDim.x) {
      const int r = i % nr, c = i / nr;
      const fcx v = sD[r + c * ld];
      dcx xv = x[r + c * ld];
      xv.x = xv.x + df64(v.x, 0.f);
      xv.y = xv.y + df64(v.y, 0.f);
      x[r + c * ld] = xv;
    }
    __syncthreads();
  }
  for (int j = L; j >= 0; --j) {
    const int dj = ext_dim(sys, j), dn = ext_dim(sys, j + 1);
    row_gemm<float, S>(dj, nr, dn, vf(sys, q, j), opN<float>(sD, ld), EpiStore<float>{sT, ld, mk<float>(1.f, 0.f)});
    row_gemm<float, S>(dj, nr, dj, opN<float>(mc.lu + j * mat, ld), opN<float>(sT, ld),
                       EpiCorr{sN, ld, mc.yv + j * mat, mc.xv + j * mat});
    fcx* t = sD;
    sD = sN;
    sN = t;
  }
  __syncthreads();
  return refine_again(sD, mc.xv, ld, sys.nl, nr, mc.red);   // sD holds d_0
}

// Stage 5: T_L = Re Tr[(X_0 Gamma_R)(X_0^H Gamma_L)] in df64.
template <int S>
__device__ double mixed_caroli(const MCtx& mc, const MSys& sys) {
  const int ld = mc.ld, nl = sys.nl, nr = sys.nr;
  dcx* sG = mc.sm[0];
  dcx* sP = mc.sm[1];
  dcx* sQ = mc.sm[2];
  copy_in(sG, ld, opN<df64>(mc.gs[M_GMR], ld), nr, nr);
  row_gemm<df64, S>(nl, nr, nr, opN<df64>(mc.xv, ld), opN<df64>(sG, ld), EpiStore<df64>{sP, ld, mk<df64>(1, 0)});
  copy_in(sG, ld, opN<df64>(mc.gs[M_GML], ld), nl, nl);
  row_gemm<df64, S>(nr, nl, nl, opC<df64>(mc.xv, ld), opN<df64>(sG, ld), EpiStore<df64>{sQ, ld, mk<df64>(1, 0)});
  return trace_prod_re(sP, ld, opN<df64>(sQ, ld), nl, nr, mc.red);
}

}  // namespace pf
