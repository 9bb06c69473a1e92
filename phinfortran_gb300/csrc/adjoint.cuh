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
  __device__ __forceinline__ void operator()(int r, int c, cx<double> acc) const {
    if (!tconj) {
      atomicAdd(&dst[r + (size_t)c * ld].x, s * acc.x);
      atomicAdd(&dst[r + (size_t)c * ld].y, s * acc.y);
    } else {
      atomicAdd(&dst[c + (size_t)r * ld].x, s * acc.x);
      atomicAdd(&dst[c + (size_t)r * ld].y, -s * acc.y);
    }
  }
};
struct EpiAddStore {  // C = acc + Y
  cx<double>* c;
  int ld;
  const cx<double>* y;
  int ldy;
  __device__ __forceinline__ void operator()(int r, int col, cx<double> acc) const {
    c[r + col * ld] = cadd(acc, y[r + col * ldy]);
  }
};

struct GradOut {
  cx<double>* gHd;   // [nq][L][n*n]
  cx<double>* gHdv;  // [nq][L-1][n*n]
  cx<double>* gHld;  // [nq][n*nl]   (M for dHld, n x nl)
  cx<double>* gHrd;  // [nq][n*nr]   (M for dHrd, n x nr)
};

struct GradSlabs {
  cx<double>* lu;  // (L+2) factors
  cx<double>* xs;  // (L+2) X blocks
  cx<double>* ys;  // (L+2) forward Z vectors
  cx<double>* k0;  // K_j
  cx<double>* k1;  // K_{j+1}
  size_t mat;
};

// Operand V_j of the extended system (global, FP64 input layout).
__device__ __forceinline__ Op<double> vop(const System<double>& s, int q, int j) {
  const int n = s.n, L = s.L;
  if (j == 0) return opN<double>(s.Hld + (size_t)q * s.nl * n, s.nl);
  if (j == L) return opC<double>(s.Hrd + (size_t)q * s.nr * n, s.nr);
  return opN<double>(s.Hdv + ((size_t)q * (L - 1) + (j - 1)) * n * n, n);
}
__device__ __forceinline__ Op<double> vop_h(const System<double>& s, int q, int j) {
  Op<double> o = vop(s, q, j);
  o.ct = !o.ct;
  return o;
}
__device__ __forceinline__ int xdim(const System<double>& s, int j) {
  return j == 0 ? s.nl : (j == s.L + 1 ? s.nr : s.n);
}

// Forward T and the weighted sensitivities of one point.  Lead results are
// expected in scratch (lead_pair).  Returns status bits; *trans = T.
template <int S>
__device__ int adjoint_point(const Ctx<double>& c, const System<double>& sys, int q, cx<double> zD, double w,
                             const GradSlabs& sl, const GradOut& go, double* trans) {
  using R = double;
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
                     EpiAddStore{sZ, ld, sl.ys + j * mat, ld});
    }
    // K_j = X_j W  (dj x nl)
    row_gemm<R, S>(dj, nl, nr, opN<R>(sl.xs + j * mat, ld), opN<R>(sW, ld), EpiStore<R>{kc, ld, mk<R>(1, 0)});
    if (j >= 1 && j <= L) {  // M_Hd_j = 2w K_j Z_j^H
      row_gemm<R, S>(dj, dj, nl, opN<R>(kc, ld), opC<R>(sZ, ld),
                     EpiAtomic{go.gHd + ((size_t)q * L + (j - 1)) * n * n, n, s2w, false});
    }
    if (j <= L) {  // M_V_j = 2w (K_{j+1} Z_j^H + (K_j Z_{j+1}^H)^H)  (d_{j+1} x d_j)
      const int dn = xdim(sys, j + 1);
      cx<R>* dst;
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

}  // namespace pf
