// Adjoint of the Caroli transmission with respect to the device blocks
// (FP64, one CTA per point).  No counterpart in the reference: the
// gradient of T (and of the thermal conductance built from it) with
// respect to masses, force constants and onsite energies.
//
// With the extended matrix A (layer 0 = left lead cell, 1..L device,
// L+1 = right lead cell; A_00 = gl^{-1}, A_jj = z_D - Hd_j,
// A_{L+1} = z_D - HR - Sigma_R, A_{j,j+1} = -V_j with V_0 = Hld,
// V_j = Hdv_j, V_L = Hrd^H), T = Re Tr[X_0 Gamma_R X_0^H Gamma_L] where
// X = A^{-1} E_{L+1}.  With W = Gamma_R X_0^H Gamma_L and Z = A^{-H} E_0
// (so G_{0,j} = Z_j^H), a weighted sum F = sum_p w_p T_p changes by
//   dF = sum_j Re Tr[dHd_j M_Hd_j] + Re Tr[dV_j M_V_j],
//   M_Hd_j = 2 w X_j W Z_j^H,
//   M_V_j  = 2 w (X_{j+1} W Z_j^H + (X_j W Z_{j+1}^H)^H).
// Cost per layer: block LU (2 GEMMs + inverse), X (2), Z forward (2),
// Z backward (2), K_j = X_j W (1), M (3)  -> 104 n^3 vs 40 n^3 forward.
#pragma once
#include "transport.cuh"

namespace pf {

// atomic accumulation of s*acc (or conj(s*acc) at the transposed position)
struct EpiAtomic {
  cx<double>* dst;
  int ld;
  double s;
  bool tconj;
  template <typename R>
  __device__ __forceinline__ void operator()(int r, int c, cx<R> acc) const {
    const double ax = to_d(acc.x), ay = to_d(acc.y);
    if (!tconj) {
      atomicAdd(&dst[r + (size_t)c * ld].x, s * ax);
      atomicAdd(&dst[r + (size_t)c * ld].y, s * ay);
    } else {
      atomicAdd(&dst[c + (size_t)r * ld].x, s * ax);
      atomicAdd(&dst[c + (size_t)r * ld].y, -s * ay);
    }
  }
};
template <typename R>
struct EpiAddStore {  // C = acc + Y
  cx<R>* c;
  int ld;
  const cx<R>* y;
  int ldy;
  __device__ __forceinline__ void operator()(int r, int col, cx<R> acc) const {
    c[r + col * ld] = cadd(acc, y[r + col * ldy]);
  }
};

struct GradOut {
  cx<double>* gHd;   // [nq][L][n*n]
  cx<double>* gHdv;  // [nq][L-1][n*n]
  cx<double>* gHld;  // [nq][n*nl]   (M for dHld, n x nl)
  cx<double>* gHrd;  // [nq][n*nr]   (M for dHrd, n x nr)
};

template <typename R>
struct GradSlabs {
  cx<R>* lu;  // (L+2) factors
  cx<R>* xs;  // (L+2) X blocks
  cx<R>* ys;  // (L+2) forward Z vectors
  cx<R>* k0;  // K_j
  cx<R>* k1;  // K_{j+1}
  size_t mat;
};

// Operand V_j of the extended system (global, FP64 input layout).
template <typename R>
__device__ __forceinline__ Op<R> vop(const System<R>& s, int q, int j) {
  const int n = s.n, L = s.L;
  if (j == 0) return opN<R>(s.Hld + (size_t)q * s.nl * n, s.nl);
  if (j == L) return opC<R>(s.Hrd + (size_t)q * s.nr * n, s.nr);
  return opN<R>(s.Hdv + ((size_t)q * (L - 1) + (j - 1)) * n * n, n);
}
template <typename R>
__device__ __forceinline__ Op<R> vop_h(const System<R>& s, int q, int j) {
  Op<R> o = vop(s, q, j);
  o.ct = !o.ct;
  return o;
}
template <typename R>
__device__ __forceinline__ int xdim(const System<R>& s, int j) {
  return j == 0 ? s.nl : (j == s.L + 1 ? s.nr : s.n);
}

// Forward T and the weighted sensitivities of one point.  Lead results are
// expected in scratch (lead_pair).  Returns status bits; *trans = T.
template <typename R, int S>
__device__ int adjoint_point(const Ctx<R>& c, const System<R>& sys, int q, cx<R> zD, double w,
                             const GradSlabs<R>& sl, const GradOut& go, double* trans) {
  const int ld = c.ld, L = sys.L, n = sys.n, nl = sys.nl, nr = sys.nr;
  const size_t mat = sl.mat;
  int st = PF_OK;
  cx<R>* s0 = c.sm[0];
  cx<R>* s1 = c.sm[1];
  cx<R>* s2 = c.sm[2];
  cx<R>* s3 = c.sm[3];
  Op<R> none = opN<R>(nullptr, 1);
  // ---- block LU: g_0 = gl, g_j = inv(A_jj - V^H g_{j-1} V)
  copy_in(sl.lu, ld, opN<R>(c.gs[G_GL], ld), nl, nl);
  for (int j = 1; j <= L + 1; ++j) {
    const int dp = xdim(sys, j - 1), dj = xdim(sys, j);
    copy_in(s0, ld, vop(sys, q, j - 1), dp, dj);
    row_gemm<R, S>(dp, dj, dp, opN<R>(sl.lu + (j - 1) * mat, ld), opN<R>(s0, ld), EpiStore<R>{s1, ld, mk<R>(1, 0)});
    EpiShift<R> e;
    e.c = s2;
    e.ld = ld;
    e.z = zD;
    if (j <= L) {
      e.h = opN<R>(sys.Hd + ((size_t)q * L + (j - 1)) * n * n, n);
      e.has_h = true;
      e.s = none;
      e.has_s = false;
    } else {
      e.h = opN<R>(sys.HR + (size_t)q * nr * nr, nr);
      e.has_h = true;
      e.s = opN<R>(c.gs[G_SR], ld);
      e.has_s = true;
    }
    row_gemm<R, S>(dj, dj, dp, opC<R>(s0, ld), opN<R>(s1, ld), e);
    st |= inverse(s2, ld, dj, c.iw);
    copy_out(sl.lu + j * mat, ld, false, s2, ld, dj, dj);
  }
  // ---- X = A^{-1} E_{L+1}: X_{L+1} = g_{L+1}, X_j = g_j V_j X_{j+1}
  copy_in(s3, ld, opN<R>(sl.lu + (L + 1) * mat, ld), nr, nr);
  copy_out(sl.xs + (L + 1) * mat, ld, false, s3, ld, nr, nr);
  for (int j = L; j >= 0; --j) {
    const int dj = xdim(sys, j), dn = xdim(sys, j + 1);
    row_gemm<R, S>(dj, nr, dn, vop(sys, q, j), opN<R>(s3, ld), EpiStore<R>{s1, ld, mk<R>(1, 0)});
    row_gemm<R, S>(dj, nr, dj, opN<R>(sl.lu + j * mat, ld), opN<R>(s1, ld), EpiStore<R>{s3, ld, mk<R>(1, 0)});
    copy_out(sl.xs + j * mat, ld, false, s3, ld, dj, nr);
  }
  // ---- T and W = Gamma_R X_0^H Gamma_L
  copy_in(s0, ld, opN<R>(c.gs[G_GMR], ld), nr, nr);
  row_gemm<R, S>(nl, nr, nr, opN<R>(sl.xs, ld), opN<R>(s0, ld), EpiStore<R>{s1, ld, mk<R>(1, 0)});  // P
  copy_in(s2, ld, opN<R>(c.gs[G_GML], ld), nl, nl);
  row_gemm<R, S>(nr, nl, nl, opC<R>(sl.xs, ld), opN<R>(s2, ld), EpiStore<R>{s3, ld, mk<R>(1, 0)});  // Q
  *trans = trace_prod_re(s1, ld, opN<R>(s3, ld), nl, nr, c.red);
  row_gemm<R, S>(nr, nl, nr, opN<R>(s0, ld), opN<R>(s3, ld), EpiStore<R>{s2, ld, mk<R>(1, 0)});  // W
  cx<R>* sW = s2;   // W stays in s2 for the rest of the point
  // ---- Z forward: y_0 = g_0^H; y_j = g_j^H V_{j-1}^H y_{j-1}
  cx<R>* sY = s0;
  cx<R>* sT = s1;
  copy_in(sY, ld, opC<R>(sl.lu, ld), nl, nl);
  copy_out(sl.ys, ld, false, sY, ld, nl, nl);
  for (int j = 1; j <= L + 1; ++j) {
    const int dp = xdim(sys, j - 1), dj = xdim(sys, j);
    row_gemm<R, S>(dj, nl, dp, vop_h(sys, q, j - 1), opN<R>(sY, ld), EpiStore<R>{sT, ld, mk<R>(1, 0)});
    row_gemm<R, S>(dj, nl, dj, opC<R>(sl.lu + j * mat, ld), opN<R>(sT, ld), EpiStore<R>{sY, ld, mk<R>(1, 0)});
    copy_out(sl.ys + j * mat, ld, false, sY, ld, dj, nl);
  }
  // ---- backward: z_j, K_j = X_j W, sensitivities
  // slots: sW (s2) = W, sZn = z_{j+1}, sZ = z_j, sT = temporary
  cx<R>* sZ = s3;
  cx<R>* sZn = s0;   // holds y_{L+1} = z_{L+1} after the forward loop
  cx<R>* kc = sl.k0;  // K_j
  cx<R>* kn = sl.k1;  // K_{j+1}
  const double s2w = 2.0 * w;
  for (int j = L + 1; j >= 0; --j) {
    const int dj = xdim(sys, j);
    if (j == L + 1) {
      copy_in(sZ, ld, opN<R>(sZn, ld), dj, nl);
    } else {
      const int dn = xdim(sys, j + 1);
      row_gemm<R, S>(dj, nl, dn, vop(sys, q, j), opN<R>(sZn, ld), EpiStore<R>{s1, ld, mk<R>(1, 0)});
      row_gemm<R, S>(dj, nl, dj, opC<R>(sl.lu + j * mat, ld), opN<R>(s1, ld),
                     EpiAddStore<R>{sZ, ld, sl.ys + j * mat, ld});
    }
    // K_j = X_j W  (dj x nl)
    row_gemm<R, S>(dj, nl, nr, opN<R>(sl.xs + j * mat, ld), opN<R>(sW, ld), EpiStore<R>{kc, ld, mk<R>(1, 0)});
    if (j >= 1 && j <= L) {  // M_Hd_j = 2w K_j Z_j^H
      row_gemm<R, S>(dj, dj, nl, opN<R>(kc, ld), opC<R>(sZ, ld),
                     EpiAtomic{go.gHd + ((size_t)q * L + (j - 1)) * n * n, n, s2w, false});
    }
    if (j <= L) {  // M_V_j = 2w (K_{j+1} Z_j^H + (K_j Z_{j+1}^H)^H)  (d_{j+1} x d_j)
      const int dn = xdim(sys, j + 1);
      cx<double>* dst;
      int ldd;
      bool hconj;  // V_L = Hrd^H: accumulate M_V_L^H into gHrd
      if (j == 0) {
        dst = go.gHld + (size_t)q * n * nl;
        ldd = n;
        hconj = false;
      } else if (j == L) {
        dst = go.gHrd + (size_t)q * n * nr;
        ldd = n;
        hconj = true;
      } else {
        dst = go.gHdv + ((size_t)q * (L - 1) + (j - 1)) * n * n;
        ldd = n;
        hconj = false;
      }
      row_gemm<R, S>(dn, dj, nl, opN<R>(kn, ld), opC<R>(sZ, ld), EpiAtomic{dst, ldd, s2w, hconj});
      row_gemm<R, S>(dj, dn, nl, opN<R>(kc, ld), opC<R>(sZn, ld), EpiAtomic{dst, ldd, s2w, !hconj});
    }
    // rotate: z_{j} becomes z_{j+1} of the next step; K likewise
    cx<R>* t = sZn;
    sZn = sZ;
    sZ = t;
    cx<R>* u = kn;
    kn = kc;
    kc = u;
  }
  return st;
}

// ---------------------------------------------------------------------------
// Checkpointed variant: memory O(sqrt(L)) instead of O(L) per point.
//
// Pass A (j = 0..L+1) forms the left-connected factors g_j and the forward
// vectors y_j, keeping (g_j, y_j) only at the checkpoints j = k*seg.  The
// forward vectors are the left-connected propagators, y_j = (G^L_{0,j})^H,
// so y_{L+1}^H = G_{0,L+1} = X_0 comes out of the same pass.
// Pass B walks the segments from the right: it recomputes the segment's
// g_j, y_j from its checkpoint and, layer by layer downwards, forms
// X_j = g_j V_j X_{j+1}, Z_j = y_j + g_j^H V_j Z_{j+1}, K_j = X_j W and the
// sensitivities.  Extra work over the store-all kernel: one recomputation
// of the factors and the y vectors.
// ---------------------------------------------------------------------------
template <typename R>
struct CkptSlabs {
  cx<R>* ckg;   // [K] checkpoint factors
  cx<R>* cky;   // [K] checkpoint y vectors
  cx<R>* segg;  // [seg] segment factors
  cx<R>* segy;  // [seg] segment y vectors
  cx<R>* pg;    // pass A rolling g
  cx<R>* py;    // pass A rolling y
  cx<R>* pG0;   // spare matrix (layout kept stable)
  cx<R>* W;     // Gamma_R X_0^H Gamma_L
  cx<R>* xa;    // X rolling pair
  cx<R>* xb;
  cx<R>* k0;    // K rolling pair
  cx<R>* k1;
  size_t mat;
  int seg;
};

// g_j and y_j from g_{j-1}, y_{j-1} (global).  Slots: V -> sv, g V -> sgv,
// the inverted block -> sg; y_j written to ydst, g_j to gdst (global).
template <typename R, int S>
__device__ int ckpt_step(const Ctx<R>& c, const System<R>& sys, int q, cx<R> zD, int j, const cx<R>* gprev,
                         const cx<R>* yprev, cx<R>* sv, cx<R>* sgv, cx<R>* sg, cx<R>* gdst, cx<R>* ydst) {
  const int ld = c.ld, L = sys.L, n = sys.n, nl = sys.nl, nr = sys.nr;
  const int dp = xdim(sys, j - 1), dj = xdim(sys, j);
  Op<R> none = opN<R>(nullptr, 1);
  copy_in(sv, ld, vop(sys, q, j - 1), dp, dj);
  row_gemm<R, S>(dp, dj, dp, opN<R>(gprev, ld), opN<R>(sv, ld), EpiStore<R>{sgv, ld, mk<R>(1, 0)});
  EpiShift<R> e;
  e.c = sg;
  e.ld = ld;
  e.z = zD;
  if (j <= L) {
    e.h = opN<R>(sys.Hd + ((size_t)q * L + (j - 1)) * n * n, n);
    e.has_h = true;
    e.s = none;
    e.has_s = false;
  } else {
    e.h = opN<R>(sys.HR + (size_t)q * nr * nr, nr);
    e.has_h = true;
    e.s = opN<R>(c.gs[G_SR], ld);
    e.has_s = true;
  }
  row_gemm<R, S>(dj, dj, dp, opC<R>(sv, ld), opN<R>(sgv, ld), e);
  const int st = inverse(sg, ld, dj, c.iw);
  // y_j = g_j^H (V^H y_{j-1})
  row_gemm<R, S>(dj, nl, dp, opC<R>(sv, ld), opN<R>(yprev, ld), EpiStore<R>{sgv, ld, mk<R>(1, 0)});
  row_gemm<R, S>(dj, nl, dj, opC<R>(sg, ld), opN<R>(sgv, ld), EpiStore<R>{ydst, ld, mk<R>(1, 0)});
  if (gdst) copy_out(gdst, ld, false, sg, ld, dj, dj);
  return st;
}

template <typename R, int S>
__device__ int adjoint_point_ckpt(const Ctx<R>& c, const System<R>& sys, int q, cx<R> zD, double w,
                                  const CkptSlabs<R>& sl, const GradOut& go, double* trans) {
  const int ld = c.ld, L = sys.L, n = sys.n, nl = sys.nl, nr = sys.nr;
  const size_t mat = sl.mat;
  const int seg = sl.seg;
  int st = PF_OK;
  cx<R>* s0 = c.sm[0];
  cx<R>* s1 = c.sm[1];
  cx<R>* s2 = c.sm[2];
  cx<R>* s3 = c.sm[3];
  // ---- pass A; the last segment's factors and y vectors go straight into
  //      the segment buffer, so pass B does not recompute that segment
  const int nseg = (L + 2 + seg - 1) / seg;
  const int cl = (nseg - 1) * seg;  // first layer of the last segment
  copy_in(sl.pg, ld, opN<R>(c.gs[G_GL], ld), nl, nl);
  copy_in(sl.py, ld, opC<R>(c.gs[G_GL], ld), nl, nl);
  copy_in(sl.ckg, ld, opN<R>(c.gs[G_GL], ld), nl, nl);
  copy_in(sl.cky, ld, opC<R>(c.gs[G_GL], ld), nl, nl);
  if (cl == 0) {
    copy_in(sl.segg, ld, opN<R>(c.gs[G_GL], ld), nl, nl);
    copy_in(sl.segy, ld, opC<R>(c.gs[G_GL], ld), nl, nl);
  }
  for (int j = 1; j <= L + 1; ++j) {
    const int dj = xdim(sys, j);
    // s0 = V_{j-1}, s1 = scratch, s2 = g_j; y_j -> py (its product reads s1, not py)
    st |= ckpt_step<R, S>(c, sys, q, zD, j, sl.pg, sl.py, s0, s1, s2, nullptr, s3);
    copy_out(sl.py, ld, false, s3, ld, dj, nl);
    copy_out(sl.pg, ld, false, s2, ld, dj, dj);
    if (j % seg == 0) {
      copy_out(sl.ckg + (size_t)(j / seg) * mat, ld, false, s2, ld, dj, dj);
      copy_out(sl.cky + (size_t)(j / seg) * mat, ld, false, s3, ld, dj, nl);
    }
    if (j >= cl) {
      copy_out(sl.segg + (size_t)(j - cl) * mat, ld, false, s2, ld, dj, dj);
      copy_out(sl.segy + (size_t)(j - cl) * mat, ld, false, s3, ld, dj, nl);
    }
  }
  // ---- T and W from X_0 = G^L_{0,L+1} = y_{L+1}^H (py holds y_{L+1}, nr x nl)
  copy_in(s0, ld, opN<R>(c.gs[G_GMR], ld), nr, nr);
  row_gemm<R, S>(nl, nr, nr, opC<R>(sl.py, ld), opN<R>(s0, ld), EpiStore<R>{s1, ld, mk<R>(1, 0)});  // P
  copy_in(s2, ld, opN<R>(c.gs[G_GML], ld), nl, nl);
  row_gemm<R, S>(nr, nl, nl, opN<R>(sl.py, ld), opN<R>(s2, ld), EpiStore<R>{s3, ld, mk<R>(1, 0)});  // Q
  *trans = trace_prod_re(s1, ld, opN<R>(s3, ld), nl, nr, c.red);
  row_gemm<R, S>(nr, nl, nr, opN<R>(s0, ld), opN<R>(s3, ld), EpiStore<R>{sl.W, ld, mk<R>(1, 0)});  // W
  // ---- pass B
  const double s2w = 2.0 * w;
  cx<R>* sZ = s3;
  cx<R>* sZn = s0;
  cx<R>* xc = sl.xa;
  cx<R>* xn = sl.xb;
  cx<R>* kc = sl.k0;
  cx<R>* kn = sl.k1;
  for (int k = nseg - 1; k >= 0; --k) {
    const int c0 = k * seg;
    const int e = (c0 + seg < L + 2) ? c0 + seg : L + 2;
    // recompute the segment's factors and y vectors (slots: s1, s2 and the
    // free Z slot); the last segment is still in the buffer from pass A
    if (k < nseg - 1) {
      copy_in(sl.segg, ld, opN<R>(sl.ckg + (size_t)k * mat, ld), xdim(sys, c0), xdim(sys, c0));
      copy_in(sl.segy, ld, opN<R>(sl.cky + (size_t)k * mat, ld), xdim(sys, c0), nl);
      for (int j = c0 + 1; j < e; ++j) {
        const int i = j - c0;
        st |= ckpt_step<R, S>(c, sys, q, zD, j, sl.segg + (size_t)(i - 1) * mat, sl.segy + (size_t)(i - 1) * mat,
                              s1, s2, sZ, sl.segg + (size_t)i * mat, sl.segy + (size_t)i * mat);
      }
    }
    // W is the right operand of every K_j of the segment: keep it in the
    // shared slot the recomputation used as scratch
    copy_in(s2, ld, opN<R>(sl.W, ld), nr, nl);
    for (int j = e - 1; j >= c0; --j) {
      const int dj = xdim(sys, j);
      const cx<R>* gj = sl.segg + (size_t)(j - c0) * mat;
      const cx<R>* yj = sl.segy + (size_t)(j - c0) * mat;
      if (j == L + 1) {
        copy_in(xc, ld, opN<R>(gj, ld), nr, nr);
        copy_in(sZ, ld, opN<R>(yj, ld), dj, nl);
      } else {
        const int dn = xdim(sys, j + 1);
        row_gemm<R, S>(dj, nr, dn, vop(sys, q, j), opN<R>(xn, ld), EpiStore<R>{s1, ld, mk<R>(1, 0)});
        row_gemm<R, S>(dj, nr, dj, opN<R>(gj, ld), opN<R>(s1, ld), EpiStore<R>{xc, ld, mk<R>(1, 0)});
        row_gemm<R, S>(dj, nl, dn, vop(sys, q, j), opN<R>(sZn, ld), EpiStore<R>{s1, ld, mk<R>(1, 0)});
        row_gemm<R, S>(dj, nl, dj, opC<R>(gj, ld), opN<R>(s1, ld), EpiAddStore<R>{sZ, ld, yj, ld});
      }
      row_gemm<R, S>(dj, nl, nr, opN<R>(xc, ld), opN<R>(s2, ld), EpiStore<R>{kc, ld, mk<R>(1, 0)});
      if (j >= 1 && j <= L) {
        row_gemm<R, S>(dj, dj, nl, opN<R>(kc, ld), opC<R>(sZ, ld),
                       EpiAtomic{go.gHd + ((size_t)q * L + (j - 1)) * n * n, n, s2w, false});
      }
      if (j <= L) {
        const int dn = xdim(sys, j + 1);
        cx<double>* dst;
        bool hconj;
        if (j == 0) {
          dst = go.gHld + (size_t)q * n * nl;
          hconj = false;
        } else if (j == L) {
          dst = go.gHrd + (size_t)q * n * nr;
          hconj = true;
        } else {
          dst = go.gHdv + ((size_t)q * (L - 1) + (j - 1)) * n * n;
          hconj = false;
        }
        row_gemm<R, S>(dn, dj, nl, opN<R>(kn, ld), opC<R>(sZ, ld), EpiAtomic{dst, n, s2w, hconj});
        row_gemm<R, S>(dj, dn, nl, opN<R>(kc, ld), opC<R>(sZn, ld), EpiAtomic{dst, n, s2w, !hconj});
      }
      cx<R>* t = sZn;
      sZn = sZ;
      sZ = t;
      cx<R>* u = xn;
      xn = xc;
      xc = u;
      cx<R>* v = kn;
      kn = kc;
      kc = v;
    }
  }
  return st;
}

}  // namespace pf
