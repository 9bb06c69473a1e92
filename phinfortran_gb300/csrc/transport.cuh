// Per-point NEGF transport pipeline: Lopez-Sancho decimation, block RGF
// sweeps and Caroli traces, executed by one CTA per (omega, q) point.
//
// Reference algorithm (KitchenSong/phinfortran):
//   decimation      negf/surface.f90:385-605 (tb/surface.f90:129-343)
//   RGF + Caroli    negf/lesser.f90:475-809  (tb/device.f90:291-575)
//
// Memory plan per CTA.  Shared memory holds the four matrices that are read
// O(n^3) times as right-hand GEMM operands or inverted in place (SM0..SM3).
// A per-CTA global scratch region (L2 resident) holds matrices that are only
// read row-wise as left operands, written by epilogues, or touched
// elementwise, plus the six lead results of the current point.
#pragma once
#include "cmat.cuh"

namespace pf {

// Block-tridiagonal system for one or more transverse q (column-major,
// interleaved complex, the reference's Haml/Hamlv/... arrays for one q each).
template <typename R>
struct System {
  int n, nl, nr, L, nq;
  const cx<R>* HL;   // [nq][nl*nl]  Haml
  const cx<R>* HLv;  // [nq][nl*nl]  Hamlv = H_{-1,0}
  const cx<R>* HR;   // [nq][nr*nr]  Hamr
  const cx<R>* HRv;  // [nq][nr*nr]  Hamrv = H_{N+2,N+1}
  const cx<R>* Hd;   // [nq][L][n*n] Hamd
  const cx<R>* Hdv;  // [nq][L-1][n*n] Hamdv = H_{i,i+1}
  const cx<R>* Hld;  // [nq][nl*n]   Hamld = H_{0,1}
  const cx<R>* Hrd;  // [nq][nr*n]   Hamrd = H_{N+1,N}
};

struct Points {
  int npts;
  const double* E;       // energy (omega^2 for phonons)
  const int* qidx;       // q index per point (nullptr: all 0)
  const int* zero_flag;  // nonzero: force T=0 (reference ie==1 rule); may be null
};

struct Params {
  const int* lead_mirror;  // per q: 1 when HR == HL and HRv == HLv bitwise (may be null)
  double eta, eta0;     // lead broadening eps = E*eta + eta0
  double dev_factor;    // device broadening multiplier (10: phonon tdb, 1: tb)
  double convergence;   // decimation stop: maxval|alpha| <= convergence
  int max_iter;         // decimation iteration cap
  int want_transr;      // also run the right-to-left sweep (T_R)
};

struct Outputs {
  double* transl;  // [npts]
  double* transr;  // [npts] (may be null when !want_transr)
  int* status;     // [npts]
  int* iters;      // [npts][2] left/right decimation iterations (may be null)
};

// Per-CTA global scratch: NG matrices of cap elements each.
enum { G_E1 = 0, G_ES, G_W2, G_W3, G_GL, G_GML, G_SL, G_GR, G_GMR, G_SR, NG };
enum { NSM = 4 };  // shared-memory slots

template <typename R>
struct Ctx {
  cx<R>* sm[NSM];
  cx<R>* gs[NG];
  int ld;  // odd leading dimension used for every working matrix
  InvWork<R> iw;
  double* red;
};

// ----------------------------------------------------------------------------
// Lopez-Sancho decimation (surface.f90:479-497).  On return SM[2] holds
// g = inv(z - es).  a0/b0 are the initial alpha/beta operands.
// ----------------------------------------------------------------------------
template <typename R, int S>
__device__ int decimate(const Ctx<R>& c, int m, cx<R> z, Op<R> h00, Op<R> a0, Op<R> b0,
                        double conv, int max_iter, int* iters_out) {
  const int ld = c.ld;
  cx<R>* al = c.sm[0];
  cx<R>* be = c.sm[1];
  cx<R>* W1 = c.sm[2];
  cx<R>* e1 = c.gs[G_E1];
  cx<R>* es = c.gs[G_ES];
  cx<R>* W2 = c.gs[G_W2];
  cx<R>* W3 = c.gs[G_W3];
  int st = PF_OK;
  copy_in(e1, ld, h00, m, m);
  copy_in(es, ld, h00, m, m);
  copy_in(al, ld, a0, m, m);
  copy_in(be, ld, b0, m, m);
  double maxdiff = max_abs(al, ld, m, m, c.red);
  int it = 0;
  while (maxdiff > conv) {
    if (it >= max_iter) {
      st |= PF_NOT_CONVERGED;
      break;
    }
    shift_neg(W1, ld, z, e1, ld, m);                      // W1 = z - e1
    st |= inverse(W1, ld, m, c.iw);                       // ive
    row_gemm<R, S>(m, m, m, opN<R>(al, ld), opN<R>(W1, ld),
                   EpiStore<R>{W2, ld, mk<R>(1, 0)});     // A = alpha ive
    row_gemm<R, S>(m, m, m, opN<R>(be, ld), opN<R>(W1, ld),
                   EpiStore<R>{W3, ld, mk<R>(1, 0)});     // B = beta ive
    row_gemm<R, S>(m, m, m, opN<R>(W2, ld), opN<R>(be, ld),
                   EpiAcc2<R>{e1, es, ld});               // e1, es += A beta
    row_gemm<R, S>(m, m, m, opN<R>(W3, ld), opN<R>(al, ld),
                   EpiAcc<R>{e1, ld});                    // e1 += B alpha
    row_gemm<R, S>(m, m, m, opN<R>(W2, ld), opN<R>(al, ld),
                   EpiStore<R>{W2, ld, mk<R>(1, 0)});     // W2 = A alpha (row in place)
    row_gemm<R, S>(m, m, m, opN<R>(W3, ld), opN<R>(be, ld),
                   EpiStore<R>{W3, ld, mk<R>(1, 0)});     // W3 = B beta (row in place)
    copy_in(al, ld, opN<R>(W2, ld), m, m);                // alpha' ; beta'
    copy_in(be, ld, opN<R>(W3, ld), m, m);
    maxdiff = max_abs(al, ld, m, m, c.red);
    ++it;
  }
  if (maxdiff != maxdiff) st |= PF_NAN;
  shift_neg(W1, ld, z, es, ld, m);
  st |= inverse(W1, ld, m, c.iw);
  if (iters_out) *iters_out = it;
  return st;
}

// Sigma = V^H g V for the lead coupling V (m x m, global), g in SM[2].
// Result in SM[1]; SM[0] holds V, G_W2 holds g V.
template <typename R, int S>
__device__ void lead_sigma(const Ctx<R>& c, int m, const cx<R>* V) {
  const int ld = c.ld;
  copy_in(c.sm[0], ld, opN<R>(V, m), m, m);
  row_gemm<R, S>(m, m, m, opN<R>(c.sm[2], ld), opN<R>(c.sm[0], ld),
                 EpiStore<R>{c.sm[3], ld, mk<R>(1, 0)});   // g V   (SM3)
  row_gemm<R, S>(m, m, m, opC<R>(c.sm[0], ld), opN<R>(c.sm[3], ld),
                 EpiStore<R>{c.sm[1], ld, mk<R>(1, 0)});   // V^H g V (SM1)
}

// dst = s * (Sig - Sig^H) with s = +i (sign>0) or -i (sign<0)
template <typename R>
__device__ void gamma_from_sigma(cx<R>* dst, int ldd, const cx<R>* Sg, int lds, int m, int sign) {
  for (int i = threadIdx.x; i < m * m; i += blockDim.x) {
    const int r = i % m, col = i / m;
    const cx<R> a = Sg[r + col * lds];
    const cx<R> b = Sg[col + r * lds];
    const cx<R> d = mk<R>(a.x - b.x, a.y + b.y);  // a - conj(b)
    dst[r + col * ldd] = sign > 0 ? mk<R>(-d.y, d.x) : mk<R>(d.y, -d.x);
  }
  __syncthreads();
}

// Left advanced + right retarded decimations of one point; leaves the
// wrapper-converted quantities of negf/lesser.f90:141-144 in global scratch:
//   G_GL = gl_adv^H, G_GML = -gml_adv, G_SL = sl_adv^H, G_GR, G_GMR, G_SR.
template <typename R, int S>
__device__ int lead_pair(const Ctx<R>& c, const System<R>& sys, int q, double E, const Params& P,
                         int* it_l, int* it_r) {
  const int ld = c.ld;
  const int nl = sys.nl, nr = sys.nr;
  const double eps = E * P.eta + P.eta0;
  int st = PF_OK;
  // left, advanced: z = E - i eps, alpha = Hamlv^H, beta = Hamlv
  {
    const cx<R>* HL = sys.HL + (size_t)q * nl * nl;
    const cx<R>* HLv = sys.HLv + (size_t)q * nl * nl;
    st |= decimate<R, S>(c, nl, mk<R>(R(E), R(-eps)), opN<R>(HL, nl), opC<R>(HLv, nl),
                         opN<R>(HLv, nl), P.convergence, P.max_iter, it_l);
    lead_sigma<R, S>(c, nl, HLv);                         // SM1 = sl_adv
    copy_out(c.gs[G_GL], ld, true, c.sm[2], ld, nl, nl);  // gl = gl_adv^H
    copy_out(c.gs[G_SL], ld, true, c.sm[1], ld, nl, nl);  // sl = sl_adv^H
    gamma_from_sigma(c.gs[G_GML], ld, c.sm[1], ld, nl, -1);  // -i(S - S^H) = -gml_adv
  }
  // right, retarded: z = E + i eps, alpha = Hamrv^H, beta = Hamrv
  if (P.lead_mirror && P.lead_mirror[q]) {
    // Identical leads: the right retarded decimation solves the adjoint of
    // the left advanced problem (H00 hermitian, beta = alpha^H), so
    // gr_ret = gl_adv^H, sr_ret = sl_adv^H, gmr_ret = -gml_adv -- exactly the
    // wrapper-converted left quantities already in scratch.
    copy_out(c.gs[G_GR], ld, false, c.gs[G_GL], ld, nl, nl);
    copy_out(c.gs[G_SR], ld, false, c.gs[G_SL], ld, nl, nl);
    copy_out(c.gs[G_GMR], ld, false, c.gs[G_GML], ld, nl, nl);
    if (it_r) *it_r = *it_l;
  } else {
    const cx<R>* HR = sys.HR + (size_t)q * nr * nr;
    const cx<R>* HRv = sys.HRv + (size_t)q * nr * nr;
    st |= decimate<R, S>(c, nr, mk<R>(R(E), R(eps)), opN<R>(HR, nr), opC<R>(HRv, nr),
                         opN<R>(HRv, nr), P.convergence, P.max_iter, it_r);
    lead_sigma<R, S>(c, nr, HRv);                         // SM1 = sr_ret
    copy_out(c.gs[G_GR], ld, false, c.sm[2], ld, nr, nr);
    copy_out(c.gs[G_SR], ld, false, c.sm[1], ld, nr, nr);
    gamma_from_sigma(c.gs[G_GMR], ld, c.sm[1], ld, nr, +1);  // i(S - S^H) = gmr_ret
  }
  return st;
}

// ----------------------------------------------------------------------------
// Left-to-right sweep + Caroli T_L (lesser.f90:547-654, 787-800).
// Slots: SM0 = V, SM1 = T, SM2 = A (inverted), SM3 = g; G_W2 = G0N, G_W3 = U.
// ----------------------------------------------------------------------------
template <typename R, int S>
__device__ int sweep_lr(const Ctx<R>& c, const System<R>& sys, int q, cx<R> zD, double* trans,
                        cx<R>* out_glr = nullptr, cx<R>* out_gr = nullptr, int ldo = 0) {
  const int ld = c.ld;
  const int n = sys.n, nl = sys.nl, nr = sys.nr, L = sys.L;
  cx<R>* V = c.sm[0];
  cx<R>* T = c.sm[1];
  cx<R>* A = c.sm[2];
  cx<R>* g = c.sm[3];
  cx<R>* G0N = c.gs[G_W2];
  cx<R>* U = c.gs[G_W3];
  const cx<R>* Hd = sys.Hd + (size_t)q * L * n * n;
  const cx<R>* Hdv = sys.Hdv + (size_t)q * (L > 1 ? L - 1 : 0) * n * n;
  const cx<R>* Hld = sys.Hld + (size_t)q * nl * n;
  const cx<R>* Hrd = sys.Hrd + (size_t)q * nr * n;
  const cx<R>* HR = sys.HR + (size_t)q * nr * nr;
  int st = PF_OK;
  Op<R> none = opN<R>(nullptr, 1);
  // layer 1: g1 = inv(zD - H1 - Hld^H gl Hld); G01 = gl Hld g1
  copy_in(A, ld, opN<R>(c.gs[G_GL], ld), nl, nl);         // gl (nl x nl)
  copy_in(V, ld, opN<R>(Hld, nl), nl, n);                 // V = Hld
  row_gemm<R, S>(nl, n, nl, opN<R>(A, ld), opN<R>(V, ld), EpiStore<R>{T, ld, mk<R>(1, 0)});
  row_gemm<R, S>(n, n, nl, opC<R>(V, ld), opN<R>(T, ld),
                 EpiShift<R>{g, ld, zD, opN<R>(Hd, n), true, none, false});
  st |= inverse(g, ld, n, c.iw);
  row_gemm<R, S>(nl, n, n, opN<R>(T, ld), opN<R>(g, ld), EpiStore<R>{G0N, ld, mk<R>(1, 0)});
  for (int i = 1; i < L; ++i) {
    copy_in(V, ld, opN<R>(Hdv + (size_t)(i - 1) * n * n, n), n, n);
    row_gemm<R, S>(n, n, n, opN<R>(g, ld), opN<R>(V, ld), EpiStore<R>{T, ld, mk<R>(1, 0)});
    row_gemm<R, S>(n, n, n, opC<R>(V, ld), opN<R>(T, ld),
                   EpiShift<R>{A, ld, zD, opN<R>(Hd + (size_t)i * n * n, n), true, none, false});
    st |= inverse(A, ld, n, c.iw);
    row_gemm<R, S>(nl, n, n, opN<R>(G0N, ld), opN<R>(V, ld), EpiStore<R>{U, ld, mk<R>(1, 0)});
    row_gemm<R, S>(nl, n, n, opN<R>(U, ld), opN<R>(A, ld), EpiStore<R>{G0N, ld, mk<R>(1, 0)});
    cx<R>* t = g;
    g = A;
    A = t;
  }
  // right closure: G_{N+1,N+1} = inv(zD - Hr - sr - Hrd g_N Hrd^H); G_{0,N+1} = G0N Hrd^H G
  copy_in(V, ld, opN<R>(Hrd, nr), nr, n);                 // V = Hrd (nr x n)
  row_gemm<R, S>(n, nr, n, opN<R>(g, ld), opC<R>(V, ld), EpiStore<R>{T, ld, mk<R>(1, 0)});
  row_gemm<R, S>(nr, nr, n, opN<R>(V, ld), opN<R>(T, ld),
                 EpiShift<R>{A, ld, zD, opN<R>(HR, nr), true, opN<R>(c.gs[G_SR], ld), true});
  st |= inverse(A, ld, nr, c.iw);
  row_gemm<R, S>(nl, nr, n, opN<R>(G0N, ld), opC<R>(V, ld), EpiStore<R>{U, ld, mk<R>(1, 0)});
  row_gemm<R, S>(nl, nr, nr, opN<R>(U, ld), opN<R>(A, ld), EpiStore<R>{T, ld, mk<R>(1, 0)});
  // T now holds G_D_LR = G_{0,N+1} (nl x nr), A holds G_R = G_{N+1,N+1}
  if (out_glr) copy_out(out_glr, ldo, false, T, ld, nl, nr);
  if (out_gr) copy_out(out_gr, ldo, false, A, ld, nr, nr);
  // Caroli: Re Tr[(G gmr)(G^H gml)]
  copy_in(A, ld, opN<R>(c.gs[G_GMR], ld), nr, nr);
  row_gemm<R, S>(nl, nr, nr, opN<R>(T, ld), opN<R>(A, ld), EpiStore<R>{U, ld, mk<R>(1, 0)});
  copy_in(A, ld, opN<R>(c.gs[G_GML], ld), nl, nl);
  row_gemm<R, S>(nr, nl, nl, opC<R>(T, ld), opN<R>(A, ld), EpiStore<R>{g, ld, mk<R>(1, 0)});
  *trans = trace_prod_re(U, ld, opN<R>(g, ld), nl, nr, c.red);
  return st;
}

// ----------------------------------------------------------------------------
// Right-to-left sweep + Caroli T_R (lesser.f90:694-793).
// ----------------------------------------------------------------------------
template <typename R, int S>
__device__ int sweep_rl(const Ctx<R>& c, const System<R>& sys, int q, cx<R> zD, double* trans,
                        cx<R>* out_grl = nullptr, cx<R>* out_gl = nullptr, int ldo = 0) {
  const int ld = c.ld;
  const int n = sys.n, nl = sys.nl, nr = sys.nr, L = sys.L;
  cx<R>* V = c.sm[0];
  cx<R>* T = c.sm[1];
  cx<R>* A = c.sm[2];
  cx<R>* g = c.sm[3];
  cx<R>* GNo = c.gs[G_W2];
  cx<R>* U = c.gs[G_W3];
  const cx<R>* Hd = sys.Hd + (size_t)q * L * n * n;
  const cx<R>* Hdv = sys.Hdv + (size_t)q * (L > 1 ? L - 1 : 0) * n * n;
  const cx<R>* Hld = sys.Hld + (size_t)q * nl * n;
  const cx<R>* Hrd = sys.Hrd + (size_t)q * nr * n;
  const cx<R>* HL = sys.HL + (size_t)q * nl * nl;
  int st = PF_OK;
  Op<R> none = opN<R>(nullptr, 1);
  // layer N: gN = inv(zD - HN - Hrd^H gr Hrd); G_{N+1,N} = gr Hrd gN
  copy_in(A, ld, opN<R>(c.gs[G_GR], ld), nr, nr);
  copy_in(V, ld, opN<R>(Hrd, nr), nr, n);
  row_gemm<R, S>(nr, n, nr, opN<R>(A, ld), opN<R>(V, ld), EpiStore<R>{T, ld, mk<R>(1, 0)});
  row_gemm<R, S>(n, n, nr, opC<R>(V, ld), opN<R>(T, ld),
                 EpiShift<R>{g, ld, zD, opN<R>(Hd + (size_t)(L - 1) * n * n, n), true, none, false});
  st |= inverse(g, ld, n, c.iw);
  row_gemm<R, S>(nr, n, n, opN<R>(T, ld), opN<R>(g, ld), EpiStore<R>{GNo, ld, mk<R>(1, 0)});
  for (int i = L - 1; i >= 1; --i) {
    // coupling V_{n+1,n} = Hamdv(i)^H; stored as Hamdv(i) and used conjugated
    copy_in(V, ld, opN<R>(Hdv + (size_t)(i - 1) * n * n, n), n, n);
    row_gemm<R, S>(n, n, n, opN<R>(g, ld), opC<R>(V, ld), EpiStore<R>{T, ld, mk<R>(1, 0)});
    row_gemm<R, S>(n, n, n, opN<R>(V, ld), opN<R>(T, ld),
                   EpiShift<R>{A, ld, zD, opN<R>(Hd + (size_t)(i - 1) * n * n, n), true, none, false});
    st |= inverse(A, ld, n, c.iw);
    row_gemm<R, S>(nr, n, n, opN<R>(GNo, ld), opC<R>(V, ld), EpiStore<R>{U, ld, mk<R>(1, 0)});
    row_gemm<R, S>(nr, n, n, opN<R>(U, ld), opN<R>(A, ld), EpiStore<R>{GNo, ld, mk<R>(1, 0)});
    cx<R>* t = g;
    g = A;
    A = t;
  }
  // left closure: G_00 = inv(zD - Hl - sl - Hld g1 Hld^H); G_{N+1,0} = GNo Hld^H G_00
  copy_in(V, ld, opN<R>(Hld, nl), nl, n);
  row_gemm<R, S>(n, nl, n, opN<R>(g, ld), opC<R>(V, ld), EpiStore<R>{T, ld, mk<R>(1, 0)});
  row_gemm<R, S>(nl, nl, n, opN<R>(V, ld), opN<R>(T, ld),
                 EpiShift<R>{A, ld, zD, opN<R>(HL, nl), true, opN<R>(c.gs[G_SL], ld), true});
  st |= inverse(A, ld, nl, c.iw);
  row_gemm<R, S>(nr, nl, n, opN<R>(GNo, ld), opC<R>(V, ld), EpiStore<R>{U, ld, mk<R>(1, 0)});
  row_gemm<R, S>(nr, nl, nl, opN<R>(U, ld), opN<R>(A, ld), EpiStore<R>{T, ld, mk<R>(1, 0)});
  // T = G_D_RL (nr x nl), A = G_L = G_{0,0}
  if (out_grl) copy_out(out_grl, ldo, false, T, ld, nr, nl);
  if (out_gl) copy_out(out_gl, ldo, false, A, ld, nl, nl);
  // Caroli: Re Tr[(G gml)(G^H gmr)]
  copy_in(A, ld, opN<R>(c.gs[G_GML], ld), nl, nl);
  row_gemm<R, S>(nr, nl, nl, opN<R>(T, ld), opN<R>(A, ld), EpiStore<R>{U, ld, mk<R>(1, 0)});
  copy_in(A, ld, opN<R>(c.gs[G_GMR], ld), nr, nr);
  row_gemm<R, S>(nl, nr, nr, opC<R>(T, ld), opN<R>(A, ld), EpiStore<R>{g, ld, mk<R>(1, 0)});
  *trans = trace_prod_re(U, ld, opN<R>(g, ld), nr, nl, c.red);
  return st;
}

}  // namespace pf
