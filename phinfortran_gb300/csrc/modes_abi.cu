// extern "C" entry of the mode-resolved transmission
// (negf/velocity_mat.f90:1692-3148 vel_mat_tdb, called per (ie, ik) from
// negf/phinfortran.f90:1238-1250), FP64.
//
// Three launches per chunk of points:
//   prep_kernel  : the four lead decimations of surface_green_tdb
//                  (surface.f90:479-593), both RGF sweeps with G_D_LR, G_R,
//                  G_D_RL, G_L kept (lesser.f90:547-784) and the Caroli T;
//                  one CTA per point, persistent.
//   lead_kernel  : one CTA per (point, lead problem) for the four transfer
//                  matrices F = g H_v: Schur form, eigenvectors, the
//                  propagating set |(|lambda| - 1)| < lambda_eta, Gram-Schmidt
//                  of the propagating columns, unfolding labels, inv(U) or
//                  inv(U^H), velocity matrix V and sqrtm(V).
//   tr_kernel    : one CTA per point: Q_L, Q_R, the t/r matrices of
//                  velocity_mat.f90:2940-2963 and the specular /
//                  non-specular sums of velocity_mat.f90:3035-3106.
#include <cuda_runtime.h>
#include <stdio.h>

#include "../../include/phinfortran_gb300.h"
#include "modes.cuh"
#include "transport.cuh"

using pf::cx;
using pf::modes::C;

namespace {

thread_local char g_err[512] = "";
int set_err(int code, const char* msg) {
  snprintf(g_err, sizeof(g_err), "%s", msg);
  return code;
}
int cuda_err(cudaError_t e, const char* where) {
  snprintf(g_err, sizeof(g_err), "%s: %s", where, cudaGetErrorString(e));
  return PF_ERR_CUDA;
}
#define MD_CUDA(call)                                  \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_err(e_, #call); \
  } while (0)

constexpr int kPrepThreads = 256;
constexpr int kTaskThreads = 128;
constexpr int kChunk = 1024;

// per-point record: matrices of ld*m elements
enum { R_GLA = 0, R_GLP, R_GRR, R_GRM, R_GML, R_GMR, R_GDLR, R_GR, R_GDRL, R_GL, NREC };
// per-task outputs: inverse eigenvector matrix and sqrtm(V)
enum { T_UINV = 0, T_VH, NTASKMAT };
enum { K_ADV_L = 0, K_RET_L, K_RET_R, K_ADV_R };

struct MLayout {
  int m, ld;
  size_t mat;        // elements per matrix
  size_t prep_smem;  // dynamic smem of prep_kernel
  size_t task_smem;  // dynamic smem of lead_kernel / tr_kernel
  size_t per_point;  // bytes of record + task outputs per point
  size_t per_cta;    // prep scratch per persistent CTA
};

MLayout mlayout(int n, int nl, int nr) {
  MLayout l;
  l.m = n > nl ? n : nl;
  l.m = l.m > nr ? l.m : nr;
  l.ld = l.m | 1;
  l.mat = (size_t)l.ld * l.m;
  l.prep_smem = pf::NSM * l.mat * 16 + 32 * sizeof(double) + 2 * (size_t)l.m * 16 + (size_t)l.m * 4 + 64 * 4;
  l.task_smem = 4 * l.mat * 16 + 32 * sizeof(double) + 3 * (size_t)l.m * 16 + 2 * (size_t)l.m * 4 + 64 * 4;
  l.per_point = ((NREC + 4 * NTASKMAT) * l.mat * 16 + 4 * (size_t)l.m * 4 + 64 + 255) & ~(size_t)255;
  l.per_cta = (size_t)pf::NG * l.mat * 16;
  return l;
}

struct Chunk {
  char* base;  // per-point records of this chunk
  size_t per_point;
  size_t mat;
  __device__ C* rec(int p, int k) const {
    return reinterpret_cast<C*>(base + (size_t)p * per_point) + (size_t)k * mat;
  }
  __device__ C* task(int p, int kind, int k) const {
    return reinterpret_cast<C*>(base + (size_t)p * per_point) + (size_t)(NREC + kind * NTASKMAT + k) * mat;
  }
  __device__ int* bz(int p, int kind, int m) const {
    return reinterpret_cast<int*>(reinterpret_cast<C*>(base + (size_t)p * per_point) +
                                  (size_t)(NREC + 4 * NTASKMAT) * mat) +
           kind * m;
  }
  __device__ int* misc(int p, int m) const {  // [4] nprop, [4] task status
    return bz(p, 0, m) + 4 * m;
  }
};

struct ModeGeom {
  double lambda_eta, a_z_l, a_z_r;
  // electron normalisation (tb/velocity_mat.f90:467, :1352-1370): V = U^H Gamma U
  // and t = i V^1/2 ... with no a_z / (2 sqrt(E)) and no 2 sqrt(E / a a)
  // factors; for E > 0 the two scalings cancel in t, r (same sums), and for
  // E <= 0 only this one is defined
  int electron;
  int nshift;
  int stride_l, nrep_l, stride_r, nrep_r;
  const cx<double>* phase_l;  // [nq][nshift][nl]
  const cx<double>* phase_r;  // [nq][nshift][nr]
};

struct ModeOut {
  double* transl;
  double* transr;
  double* sums;  // [npts][8]
  int* status;
  int* nprop;    // [npts][4] or null
  // per-mode outputs (all null, or all set):
  double* mode_kz;   // [npts][4 problems][mm] k_z of every mode, 100 when not propagating
  int* mode_bz;      // [npts][4 problems][mm] unfolding label (0: not propagating)
  double* col_sums;  // [npts][4 matrices][mm columns][nshift] sum of |M_rc|^2 over the rows of each label
  int mm;            // max(nl, nr)
  double* md2md;     // [npts][4 matrices][mm columns][mm rows] |M_rc|^2 (nullable)
};

// reference value of pi (negf/util.f90:5)
constexpr double kPi = 3.141592653589793238;

__device__ void make_ctx_prep(pf::Ctx<double>& c, const MLayout& lay, char* gscr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<double>* s = reinterpret_cast<cx<double>*>(smem_raw);
  for (int i = 0; i < pf::NSM; ++i) c.sm[i] = s + i * lay.mat;
  unsigned char* tail = reinterpret_cast<unsigned char*>(s + pf::NSM * lay.mat);
  c.red = reinterpret_cast<double*>(tail);
  c.iw.rowk = reinterpret_cast<cx<double>*>(tail + 32 * sizeof(double));
  c.iw.colk = c.iw.rowk + lay.m;
  int* ip = reinterpret_cast<int*>(c.iw.colk + lay.m);
  c.iw.perm = ip;
  c.iw.flag = ip + lay.m;
  cx<double>* g = reinterpret_cast<cx<double>*>(gscr) + (size_t)blockIdx.x * pf::NG * lay.mat;
  for (int i = 0; i < pf::NG; ++i) c.gs[i] = g + i * lay.mat;
  c.ld = lay.ld;
}

template <int S>
__global__ void __launch_bounds__(kPrepThreads)
    prep_kernel(pf::System<double> sys, pf::Points pts, int p0, int cnt, pf::Params P, MLayout lay, Chunk ch,
                char* gscr, int* queue, ModeOut out) {
  pf::Ctx<double> c;
  make_ctx_prep(c, lay, gscr);
  const int ld = lay.ld;
  const int nl = sys.nl, nr = sys.nr;
  __shared__ int s_p;
  for (;;) {
    if (threadIdx.x == 0) s_p = atomicAdd(queue, 1);
    __syncthreads();
    const int lp = s_p;
    __syncthreads();
    if (lp >= cnt) break;
    const int p = p0 + lp;
    const int q = pts.qidx ? pts.qidx[p] : 0;
    const double E = pts.E[p];
    int itl = 0, itr = 0;
    int st = pf::lead_pair<double, S>(c, sys, q, E, P, &itl, &itr);
    // raw surface outputs as vel_mat_tdb receives them
    pf::copy_out(ch.rec(lp, R_GLA), ld, true, c.gs[pf::G_GL], ld, nl, nl);    // gl_adv
    pf::copy_out(ch.rec(lp, R_GRR), ld, false, c.gs[pf::G_GR], ld, nr, nr);   // gr_ret
    pf::copy_out(ch.rec(lp, R_GMR), ld, false, c.gs[pf::G_GMR], ld, nr, nr);  // gmr_ret
    {
      C* d = ch.rec(lp, R_GML);  // gml_adv = -(converted)
      const C* s = c.gs[pf::G_GML];
      for (int i = threadIdx.x; i < nl * nl; i += blockDim.x) {
        const int r = i % nl, cc = i / nl;
        const C v = s[r + cc * ld];
        d[r + cc * ld] = pf::mk<double>(-v.x, -v.y);
      }
      __syncthreads();
    }
    const double eps = E * P.eta + P.eta0;
    // left "plus" (surface.f90:510-532): z = E + i eps, alpha = Hamlv, beta = Hamlv^H
    {
      const C* HL = sys.HL + (size_t)q * nl * nl;
      const C* HLv = sys.HLv + (size_t)q * nl * nl;
      st |= pf::decimate<double, S>(c, nl, pf::mk<double>(E, eps), pf::opN<double>(HL, nl),
                                    pf::opN<double>(HLv, nl), pf::opC<double>(HLv, nl), P.convergence, P.max_iter,
                                    nullptr);
      pf::copy_out(ch.rec(lp, R_GLP), ld, false, c.sm[2], ld, nl, nl);
    }
    // right "minus" (surface.f90:571-593): z = E - i eps, alpha = Hamrv, beta = Hamrv^H.
    // Identical leads: the adjoint of the left "plus" problem, gr_minus = gl_plus^H
    // (the relation lead_pair uses for gr_ret = gl_adv^H).
    if (P.lead_mirror && P.lead_mirror[q]) {
      pf::copy_out(ch.rec(lp, R_GRM), ld, true, ch.rec(lp, R_GLP), ld, nr, nr);
    } else {
      const C* HR = sys.HR + (size_t)q * nr * nr;
      const C* HRv = sys.HRv + (size_t)q * nr * nr;
      st |= pf::decimate<double, S>(c, nr, pf::mk<double>(E, -eps), pf::opN<double>(HR, nr),
                                    pf::opN<double>(HRv, nr), pf::opC<double>(HRv, nr), P.convergence, P.max_iter,
                                    nullptr);
      pf::copy_out(ch.rec(lp, R_GRM), ld, false, c.sm[2], ld, nr, nr);
    }
    const cx<double> zD = pf::mk<double>(E, P.dev_factor * eps);
    double tl = 0, tr = 0;
    st |= pf::sweep_lr<double, S>(c, sys, q, zD, &tl, ch.rec(lp, R_GDLR), ch.rec(lp, R_GR), ld);
    st |= pf::sweep_rl<double, S>(c, sys, q, zD, &tr, ch.rec(lp, R_GDRL), ch.rec(lp, R_GL), ld);
    if (threadIdx.x == 0) {
      const bool zero = pts.zero_flag && pts.zero_flag[p];
      double a = tl, b = tr;
      if (zero || a < 1.0e-60) a = 0.0;
      if (zero || b < 1.0e-60) b = 0.0;
      out.transl[p] = a;
      if (out.transr) out.transr[p] = b;
      out.status[p] = st;
    }
    __syncthreads();
  }
}

struct TaskSmem {
  C* s[4];
  C* v;
  C* rowk;
  C* colk;
  double* red;
  int* cols;
  int* perm;
  int* flag;
};

__device__ TaskSmem task_smem(const MLayout& lay) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TaskSmem t;
  C* s = reinterpret_cast<C*>(smem_raw);
  for (int i = 0; i < 4; ++i) t.s[i] = s + i * lay.mat;
  t.v = s + 4 * lay.mat;
  t.rowk = t.v + lay.m;
  t.colk = t.rowk + lay.m;
  t.red = reinterpret_cast<double*>(t.colk + lay.m);
  t.cols = reinterpret_cast<int*>(t.red + 32);
  t.perm = t.cols + lay.m;
  t.flag = t.perm + lay.m;
  return t;
}

template <class Epi>
__device__ void mm(int m, int n, int k, pf::Op<double> A, pf::Op<double> B, const Epi& e, int S) {
  if (S == 1)
    pf::row_gemm<double, 1>(m, n, k, A, B, e);
  else
    pf::row_gemm<double, 2>(m, n, k, A, B, e);
}

// One CTA per (point, lead problem).
__global__ void __launch_bounds__(kTaskThreads)
    lead_kernel(pf::System<double> sys, pf::Points pts, int p0, int cnt, MLayout lay, Chunk ch, ModeGeom geo,
                ModeOut out) {
  const int lp = blockIdx.x >> 2;
  const int kind = blockIdx.x & 3;
  if (lp >= cnt) return;
  const int p = p0 + lp;
  const int q = pts.qidx ? pts.qidx[p] : 0;
  const double E = pts.E[p];
  const int ld = lay.ld;
  const bool left = (kind == K_ADV_L || kind == K_RET_L);
  const int m = left ? sys.nl : sys.nr;
  const int S = (m + 31) / 32;
  TaskSmem t = task_smem(lay);
  const int tid = threadIdx.x, nt = blockDim.x;
  int st = 0;
  // ---- F = g' H_v
  const C* Hv = left ? sys.HLv + (size_t)q * m * m : sys.HRv + (size_t)q * m * m;
  const C* g = ch.rec(lp, left ? R_GLA : R_GRR);
  const bool gct = (kind == K_RET_L || kind == K_ADV_R);  // gl^H / gr^H
  pf::copy_in(t.s[1], ld, gct ? pf::opC<double>(g, ld) : pf::opN<double>(g, ld), m, m);
  pf::copy_in(t.s[2], ld, pf::opN<double>(Hv, m), m, m);
  mm(m, m, m, pf::opN<double>(t.s[1], ld), pf::opN<double>(t.s[2], ld),
     pf::EpiStore<double>{t.s[0], ld, pf::mk<double>(1, 0)}, S);
  // ---- Schur form and eigenvectors
  st |= pf::modes::schur(t.s[0], t.s[1], ld, m, t.v, t.red);
  // propagating set, in eigenvalue order
  if (tid == 0) {
    int np = 0;
    for (int i = 0; i < m; ++i) {
      const C lam = t.s[0][i + i * ld];
      if (fabs(hypot(lam.x, lam.y) - 1.0) < geo.lambda_eta) t.cols[np++] = i;
    }
    t.flag[0] = np;
  }
  __syncthreads();
  const int np = t.flag[0];
  // keep the eigenvalues of the propagating columns (diag of T) in rowk
  for (int i = tid; i < np; i += nt) t.rowk[i] = t.s[0][t.cols[i] + t.cols[i] * ld];
  pf::modes::tri_eigvecs(t.s[0], t.s[2], ld, m);
  mm(m, m, m, pf::opN<double>(t.s[1], ld), pf::opN<double>(t.s[2], ld),
     pf::EpiStore<double>{t.s[3], ld, pf::mk<double>(1, 0)}, S);
  pf::modes::normalise_columns(t.s[3], ld, m);
  if (np > 0) pf::modes::gram_schmidt_cols(t.s[3], t.s[2], ld, m, t.cols, np, t.red);
  // ---- unfolding labels (velocity_mat.f90:2035-2072)
  int* bz = ch.bz(lp, kind, lay.m);
  for (int i = tid; i < m; i += nt) bz[i] = 0;
  __syncthreads();
  {
    const int ns = geo.nshift;
    const int stride = left ? geo.stride_l : geo.stride_r;
    const int nrep = left ? geo.nrep_l : geo.nrep_r;
    const int nimg = m / stride;
    const C* ph = (left ? geo.phase_l : geo.phase_r) + (size_t)q * ns * m;
    double* w = reinterpret_cast<double*>(t.s[2]);  // np * ns doubles (slot 2 is free here)
    for (int u = tid; u < np * ns; u += nt) {
      const int ci = u / ns, js = u % ns;
      const int col = t.cols[ci];
      const C lam = t.rowk[ci];
      double acc = 0.0;
      for (int r0 = 0; r0 < nrep; ++r0) {
        C s = pf::mk<double>(0.0, 0.0);
        for (int ir = 0; ir < nimg; ++ir) {
          const int row = r0 + stride * ir;
          s = pf::cfma(pf::cmul(ph[(size_t)js * m + row], t.s[3][row + col * ld]), lam, s);
        }
        acc += (s.x * s.x + s.y * s.y) / (double)nimg;
      }
      w[u] = acc;
    }
    __syncthreads();
    for (int ci = tid; ci < np; ci += nt) {
      int best = 0;
      for (int js = 1; js < ns; ++js)
        if (w[ci * ns + js] > w[ci * ns + best]) best = js;
      bz[t.cols[ci]] = best + 1;
    }
    __syncthreads();
  }
  // ---- per-mode outputs in this kernel's mode order: the unfolding label
  //      and k_z = sign * log_fbz(lambda) (negf/util.f90:825-839; sign -1 on
  //      the left, velocity_mat.f90:2353-2360), 100 when not propagating
  if (out.mode_kz) {
    const size_t o = ((size_t)p * 4 + kind) * out.mm;
    for (int i = tid; i < m; i += nt) {
      out.mode_kz[o + i] = 100.0;
      out.mode_bz[o + i] = bz[i];
    }
    __syncthreads();
    const double az = left ? geo.a_z_l : geo.a_z_r;
    const double gz = 2.0 * kPi / az;
    for (int ci = tid; ci < np; ci += nt) {
      const C lam = t.rowk[ci];
      double kz = fmod(atan2(lam.y, lam.x) / az, gz);   // Re(log(lambda) / (i a_z)) folded
      if (kz < 0.0) kz += gz;
      if (kz > 0.5 * gz) kz -= gz;
      out.mode_kz[o + t.cols[ci]] = left ? -kz : kz;
    }
  }
  // ---- velocity matrix V = sign (U^H Gamma U) i a / (2 sqrt(E))
  const C* gam = ch.rec(lp, left ? R_GML : R_GMR);  // Hermitian: Gamma^H == Gamma bitwise
  mm(m, m, m, pf::opC<double>(gam, ld), pf::opN<double>(t.s[3], ld),
     pf::EpiStore<double>{t.s[2], ld, pf::mk<double>(1, 0)}, S);
  const double az = left ? geo.a_z_l : geo.a_z_r;
  const double sgn = left ? -1.0 : 1.0;
  const double f = geo.electron ? sgn : sgn * az / 2.0 / sqrt(E);
  mm(m, m, m, pf::opC<double>(t.s[3], ld), pf::opN<double>(t.s[2], ld),
     pf::EpiStore<double>{t.s[0], ld, pf::mk<double>(0.0, f)}, S);
  // ---- inv(U^H) (advanced problems) or inv(U) (retarded)
  const bool invh = (kind == K_ADV_L || kind == K_ADV_R);
  pf::copy_in(t.s[1], ld, invh ? pf::opC<double>(t.s[3], ld) : pf::opN<double>(t.s[3], ld), m, m);
  // the inversion reuses rowk (eigenvalues no longer needed) and v
  pf::InvWork<double> iw{t.rowk, t.v, t.perm, t.flag};
  st |= pf::inverse(t.s[1], ld, m, iw);
  pf::copy_out(ch.task(lp, kind, T_UINV), ld, false, t.s[1], ld, m, m);
  // ---- sqrtm(V): Schur form, triangular square root, Z U Z^H
  st |= pf::modes::schur(t.s[0], t.s[1], ld, m, t.v, t.red);
  pf::modes::sqrt_tri(t.s[0], t.s[2], ld, m);
  mm(m, m, m, pf::opN<double>(t.s[1], ld), pf::opN<double>(t.s[2], ld),
     pf::EpiStore<double>{t.s[3], ld, pf::mk<double>(1, 0)}, S);
  mm(m, m, m, pf::opN<double>(t.s[3], ld), pf::opC<double>(t.s[1], ld),
     pf::EpiStore<double>{ch.task(lp, kind, T_VH), ld, pf::mk<double>(1, 0)}, S);
  if (tid == 0) {
    int* misc = ch.misc(lp, lay.m);
    misc[kind] = np;
    misc[4 + kind] = st;
  }
}

struct EpiSub {  // C -= acc
  C* c;
  int ld;
  __device__ __forceinline__ void operator()(int r, int col, C acc) const {
    c[r + col * ld] = pf::csub(c[r + col * ld], acc);
  }
};

// s / ns sums of |M_ij|^2 over labelled rows and columns
__device__ void split_sums(const C* M, int ld, int rows, int cols, const int* bzr, const int* bzc, double* red,
                           double* s_out, double* ns_out) {
  double s = 0.0, ns = 0.0;
  for (int i = threadIdx.x; i < rows * cols; i += blockDim.x) {
    const int r = i % rows, c = i / rows;
    const int a = bzr[r], b = bzc[c];
    if (a <= 0 || b <= 0) continue;
    const C e = M[r + c * ld];
    const double v = e.x * e.x + e.y * e.y;
    if (a == b)
      s += v;
    else
      ns += v;
  }
  *s_out = pf::modes::block_sum(s, red);
  *ns_out = pf::modes::block_sum(ns, red);
}

// Q = (E + i eps) I - H00 - V^H gA V - V gB V^H with gA = opA, gB = opB.
__device__ void bulk_q(C* Q, C* w0, C* w1, C* w2, int ld, int m, double E, double eps, const C* H00, const C* V,
                       pf::Op<double> gA, pf::Op<double> gB, int S) {
  pf::copy_in(w0, ld, pf::opN<double>(V, m), m, m);
  pf::copy_in(w1, ld, gA, m, m);
  mm(m, m, m, pf::opN<double>(w1, ld), pf::opN<double>(w0, ld), pf::EpiStore<double>{w2, ld, pf::mk<double>(1, 0)},
     S);
  pf::Op<double> none = pf::opN<double>(nullptr, 1);
  mm(m, m, m, pf::opC<double>(w0, ld), pf::opN<double>(w2, ld),
     pf::EpiShift<double>{Q, ld, pf::mk<double>(E, eps), pf::opN<double>(H00, m), true, none, false}, S);
  pf::copy_in(w1, ld, gB, m, m);
  mm(m, m, m, pf::opN<double>(w1, ld), pf::opC<double>(w0, ld), pf::EpiStore<double>{w2, ld, pf::mk<double>(1, 0)},
     S);
  mm(m, m, m, pf::opN<double>(w0, ld), pf::opN<double>(w2, ld), EpiSub{Q, ld}, S);
}

// One CTA per point: t/r matrices and their specular / non-specular sums.
__global__ void __launch_bounds__(kTaskThreads)
    tr_kernel(pf::System<double> sys, pf::Points pts, int p0, int cnt, MLayout lay, Chunk ch, ModeGeom geo,
              double eta, double eta0, ModeOut out) {
  const int lp = blockIdx.x;
  if (lp >= cnt) return;
  const int p = p0 + lp;
  const int q = pts.qidx ? pts.qidx[p] : 0;
  const double E = pts.E[p];
  const int ld = lay.ld;
  const int nl = sys.nl, nr = sys.nr;
  const int S = (lay.m + 31) / 32;
  TaskSmem t = task_smem(lay);
  pf::InvWork<double> iw{t.rowk, t.colk, t.perm, t.flag};
  const double eps = E * eta + eta0;
  int st = 0;
  const int* misc = ch.misc(lp, lay.m);
  for (int k = 0; k < 4; ++k) st |= misc[4 + k];
  const bool zero = pts.zero_flag && pts.zero_flag[p];
  double sums[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  const C* HL = sys.HL + (size_t)q * nl * nl;
  const C* HLv = sys.HLv + (size_t)q * nl * nl;
  const C* HR = sys.HR + (size_t)q * nr * nr;
  const C* HRv = sys.HRv + (size_t)q * nr * nr;
  const int* bz_al = ch.bz(lp, K_ADV_L, lay.m);
  const int* bz_rl = ch.bz(lp, K_RET_L, lay.m);
  const int* bz_rr = ch.bz(lp, K_RET_R, lay.m);
  const int* bz_ar = ch.bz(lp, K_ADV_R, lay.m);
  // M = c * Vh_row Uinv_row X Uinv_col Vh_col, X (rows x cols) given as an Op
  // per-column sums of |M_rc|^2 grouped by the row's label (M in slot 0):
  // mat 0 tlr, 1 trl, 2 rrr, 3 rll; columns without a label stay zero
  const int nsh = geo.nshift;
  auto col_out = [&](int mat, int rows, int cols, const int* bzr, const int* bzc) {
    if (out.md2md) {
      // the whole mode-to-mode matrix |M_rc|^2 (write_md2md, negf/write_data.f90:177-241)
      double* o = out.md2md + ((size_t)p * 4 + mat) * out.mm * out.mm;
      for (int u = threadIdx.x; u < rows * cols; u += blockDim.x) {
        const int r = u % rows, c = u / rows;
        const C e = t.s[0][r + c * ld];
        o[r + (size_t)c * out.mm] = e.x * e.x + e.y * e.y;
      }
      __syncthreads();
    }
    if (!out.col_sums) return;
    double* o = out.col_sums + ((size_t)p * 4 + mat) * out.mm * nsh;
    for (int u = threadIdx.x; u < cols * nsh; u += blockDim.x) {
      const int c = u / nsh, b = u % nsh + 1;
      double acc = 0.0;
      if (bzc[c] > 0)
        for (int r = 0; r < rows; ++r)
          if (bzr[r] == b) {
            const C e = t.s[0][r + c * ld];
            acc += e.x * e.x + e.y * e.y;
          }
      o[u] = acc;
    }
    __syncthreads();
  };
  if (out.col_sums) {
    double* o = out.col_sums + (size_t)p * 4 * out.mm * nsh;
    for (int u = threadIdx.x; u < 4 * out.mm * nsh; u += blockDim.x) o[u] = 0.0;
    __syncthreads();
  }
  if (out.md2md) {
    double* o = out.md2md + (size_t)p * 4 * out.mm * out.mm;
    for (int u = threadIdx.x; u < 4 * out.mm * out.mm; u += blockDim.x) o[u] = 0.0;
    __syncthreads();
  }
  // prefactor of the t / r chains: 2 sqrt(E / (a_row a_col)) (phonons), 1 (electrons)
  auto cf = [&](double ar, double ac) { return geo.electron ? 1.0 : 2.0 * sqrt(E / ar / ac); };
  auto chain = [&](int rows, int cols, int krow, int kcol, pf::Op<double> X, double cfac) {
    // s0 = Uinv_col Vh_col (cols x cols)
    pf::copy_in(t.s[0], ld, pf::opN<double>(ch.task(lp, kcol, T_UINV), ld), cols, cols);
    pf::copy_in(t.s[1], ld, pf::opN<double>(ch.task(lp, kcol, T_VH), ld), cols, cols);
    mm(cols, cols, cols, pf::opN<double>(t.s[0], ld), pf::opN<double>(t.s[1], ld),
       pf::EpiStore<double>{t.s[2], ld, pf::mk<double>(1, 0)}, S);
    // s0 = X s2 (rows x cols)
    pf::copy_in(t.s[1], ld, X, rows, cols);
    mm(rows, cols, cols, pf::opN<double>(t.s[1], ld), pf::opN<double>(t.s[2], ld),
       pf::EpiStore<double>{t.s[0], ld, pf::mk<double>(1, 0)}, S);
    // s2 = Uinv_row s0
    pf::copy_in(t.s[1], ld, pf::opN<double>(ch.task(lp, krow, T_UINV), ld), rows, rows);
    mm(rows, cols, rows, pf::opN<double>(t.s[1], ld), pf::opN<double>(t.s[0], ld),
       pf::EpiStore<double>{t.s[2], ld, pf::mk<double>(1, 0)}, S);
    // s0 = i cfac Vh_row s2
    pf::copy_in(t.s[1], ld, pf::opN<double>(ch.task(lp, krow, T_VH), ld), rows, rows);
    mm(rows, cols, rows, pf::opN<double>(t.s[1], ld), pf::opN<double>(t.s[2], ld),
       pf::EpiStore<double>{t.s[0], ld, pf::mk<double>(0.0, cfac)}, S);
  };
  if (!zero) {
    // trl = i 2 sqrt(E/azR/azL) Vh_rR Uinv_rR G_D_RL Uinv_aL Vh_aL  -> transr
    chain(nr, nl, K_RET_R, K_ADV_L, pf::opN<double>(ch.rec(lp, R_GDRL), ld), cf(geo.a_z_r, geo.a_z_l));
    split_sums(t.s[0], ld, nr, nl, bz_rr, bz_al, t.red, &sums[2], &sums[3]);
    col_out(1, nr, nl, bz_rr, bz_al);
    // tlr = i 2 sqrt(E/azL/azR) Vh_rL Uinv_rL G_D_LR Uinv_aR Vh_aR  -> transl
    chain(nl, nr, K_RET_L, K_ADV_R, pf::opN<double>(ch.rec(lp, R_GDLR), ld), cf(geo.a_z_l, geo.a_z_r));
    split_sums(t.s[0], ld, nl, nr, bz_rl, bz_ar, t.red, &sums[0], &sums[1]);
    col_out(0, nl, nr, bz_rl, bz_ar);
    // rrr: (G_R - inv(Q_R)), Q_R = z - Hr - Hrv^H gr Hrv - Hrv grm^H Hrv^H
    bulk_q(t.s[3], t.s[0], t.s[1], t.s[2], ld, nr, E, eps, HR, HRv, pf::opN<double>(ch.rec(lp, R_GRR), ld),
           pf::opC<double>(ch.rec(lp, R_GRM), ld), S);
    st |= pf::inverse(t.s[3], ld, nr, iw);
    {
      const C* G = ch.rec(lp, R_GR);
      for (int i = threadIdx.x; i < nr * nr; i += blockDim.x) {
        const int r = i % nr, c = i / nr;
        t.s[3][r + c * ld] = pf::csub(G[r + c * ld], t.s[3][r + c * ld]);
      }
      __syncthreads();
    }
    // the chain reads X before it reuses slot 3? no: X is copied into s1 first
    chain(nr, nr, K_RET_R, K_ADV_R, pf::opN<double>(t.s[3], ld), cf(geo.a_z_r, geo.a_z_r));
    split_sums(t.s[0], ld, nr, nr, bz_rr, bz_ar, t.red, &sums[6], &sums[7]);
    col_out(2, nr, nr, bz_rr, bz_ar);
    // rll: (G_L - inv(Q_L)), Q_L = z - Hl - Hlv^H gl^H Hlv - Hlv glp Hlv^H
    bulk_q(t.s[3], t.s[0], t.s[1], t.s[2], ld, nl, E, eps, HL, HLv, pf::opC<double>(ch.rec(lp, R_GLA), ld),
           pf::opN<double>(ch.rec(lp, R_GLP), ld), S);
    st |= pf::inverse(t.s[3], ld, nl, iw);
    {
      const C* G = ch.rec(lp, R_GL);
      for (int i = threadIdx.x; i < nl * nl; i += blockDim.x) {
        const int r = i % nl, c = i / nl;
        t.s[3][r + c * ld] = pf::csub(G[r + c * ld], t.s[3][r + c * ld]);
      }
      __syncthreads();
    }
    chain(nl, nl, K_RET_L, K_ADV_L, pf::opN<double>(t.s[3], ld), cf(geo.a_z_l, geo.a_z_l));
    split_sums(t.s[0], ld, nl, nl, bz_rl, bz_al, t.red, &sums[4], &sums[5]);
    col_out(3, nl, nl, bz_rl, bz_al);
  }
  if (threadIdx.x == 0) {
    for (int k = 0; k < 8; ++k) out.sums[(size_t)p * 8 + k] = sums[k];
    out.status[p] |= st;
    if (out.nprop)
      for (int k = 0; k < 4; ++k) out.nprop[(size_t)p * 4 + k] = misc[k];
  }
}

__global__ void mirror_kernel(const double* HL, const double* HLv, const double* HR, const double* HRv, int m2,
                              int nq, int* mirror) {
  const int q = blockIdx.x;
  if (q >= nq) return;
  __shared__ int diff;
  if (threadIdx.x == 0) diff = 0;
  __syncthreads();
  const size_t off = (size_t)q * m2;
  int d = 0;
  for (int i = threadIdx.x; i < m2; i += blockDim.x)
    d |= (__double_as_longlong(HL[off + i]) != __double_as_longlong(HR[off + i])) |
         (__double_as_longlong(HLv[off + i]) != __double_as_longlong(HRv[off + i]));
  if (d) atomicOr(&diff, 1);
  __syncthreads();
  if (threadIdx.x == 0) mirror[q] = diff ? 0 : 1;
}

int prep_grid(const MLayout& lay, int npts, int S) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e;
  if (S == 1) {
    e = cudaFuncSetAttribute(prep_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.prep_smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, prep_kernel<1>, kPrepThreads, lay.prep_smem);
  } else {
    e = cudaFuncSetAttribute(prep_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.prep_smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, prep_kernel<2>, kPrepThreads, lay.prep_smem);
  }
  if (e != cudaSuccess || per_sm < 1) return -1;
  const int g = sms * per_sm;
  return g < npts ? g : npts;
}

// Packed per-point outputs of pf_transport_tdb_blocks_dev: record k of a
// chunk (leading dimension ld) -> dst[k] + p * rows[k] * cols[k]
// (column-major), for the records whose dst is set.
struct BlockOut {
  double* dst[NREC];
  int rows[NREC], cols[NREC];
};

__global__ void blocks_out_kernel(Chunk ch, int p0, int cnt, int ld, BlockOut bo) {
  const int lp = blockIdx.x, k = blockIdx.y;
  if (lp >= cnt || bo.dst[k] == nullptr) return;
  const int rows = bo.rows[k], cols = bo.cols[k];
  const C* src = ch.rec(lp, k);
  C* d = reinterpret_cast<C*>(bo.dst[k]) + (size_t)(p0 + lp) * rows * cols;
  for (int i = threadIdx.x; i < rows * cols; i += blockDim.x) d[i] = src[i % rows + (i / rows) * ld];
}

size_t modes_bytes(const MLayout& lay, int nq, int chunk, int grid) {
  const size_t mir = ((size_t)nq * 4 + 255) & ~(size_t)255;
  return 256 + mir + (size_t)grid * lay.per_cta + (size_t)chunk * lay.per_point;
}

}  // namespace

extern "C" {

const char* pf_modes_last_error(void) { return g_err; }

size_t pf_transport_tdb_modes_workspace_size(int n, int nl, int nr, int nq, int npts) {
  if (n <= 0 || nl <= 0 || nr <= 0 || nq <= 0 || npts < 0) return 0;
  if (n > PF_NMAX_RESIDENT || nl > PF_NMAX_RESIDENT || nr > PF_NMAX_RESIDENT) return 0;
  const MLayout lay = mlayout(n, nl, nr);
  const int chunk = npts < kChunk ? (npts > 0 ? npts : 1) : kChunk;
  const int grid = prep_grid(lay, chunk, (lay.m + 31) / 32);
  if (grid <= 0) return 0;
  return modes_bytes(lay, nq, chunk, grid);
}

int pf_transport_tdb_modes_ex_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                                  const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                                  const double* Hld, const double* Hrd, int npts, const double* E,
                                  const int* qidx, const int* zero_flag, double eta, double eta0,
                                  double dev_factor, double convergence, int max_iter, double lambda_eta,
                                  double a_z_l, double a_z_r, int nshift, int stride_l, int nrep_l,
                                  const double* phase_l, int stride_r, int nrep_r, const double* phase_r,
                                  int flags, double* transl, double* transr, double* mode_sums, int* status,
                                  int* nprop, double* mode_kz, int* mode_bz, double* col_sums, void* work,
                                  size_t work_bytes, void* stream) {
  return pf_transport_tdb_modes_md2md_dev(n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd, npts, E, qidx,
                                          zero_flag, eta, eta0, dev_factor, convergence, max_iter, lambda_eta,
                                          a_z_l, a_z_r, nshift, stride_l, nrep_l, phase_l, stride_r, nrep_r,
                                          phase_r, flags, transl, transr, mode_sums, status, nprop, mode_kz,
                                          mode_bz, col_sums, nullptr, work, work_bytes, stream);
}

int pf_transport_tdb_modes_md2md_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                                     const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                                     const double* Hld, const double* Hrd, int npts, const double* E,
                                     const int* qidx, const int* zero_flag, double eta, double eta0,
                                     double dev_factor, double convergence, int max_iter, double lambda_eta,
                                     double a_z_l, double a_z_r, int nshift, int stride_l, int nrep_l,
                                     const double* phase_l, int stride_r, int nrep_r, const double* phase_r,
                                     int flags, double* transl, double* transr, double* mode_sums, int* status,
                                     int* nprop, double* mode_kz, int* mode_bz, double* col_sums,
                                     double* md2md, void* work, size_t work_bytes, void* stream) {
  if (flags & ~PF_MODES_ELECTRON) return set_err(PF_ERR_ARG, "pf_modes: unknown flags");
  if (md2md && !mode_kz) return set_err(PF_ERR_ARG, "pf_modes: md2md needs the per-mode outputs");
  if ((mode_kz != nullptr) != (mode_bz != nullptr) || (mode_kz != nullptr) != (col_sums != nullptr))
    return set_err(PF_ERR_ARG, "pf_modes: mode_kz, mode_bz and col_sums are all given or all null");
  if (n <= 0 || nl <= 0 || nr <= 0 || L <= 0 || nq <= 0 || npts < 0)
    return set_err(PF_ERR_ARG, "pf_modes: dimensions must be positive");
  if (n > PF_NMAX_RESIDENT || nl > PF_NMAX_RESIDENT || nr > PF_NMAX_RESIDENT)
    return set_err(PF_ERR_SIZE, "pf_modes: block size exceeds the resident kernel limit");
  if (!HL || !HLv || !HR || !HRv || !Hd || !Hld || !Hrd || (L > 1 && !Hdv))
    return set_err(PF_ERR_ARG, "pf_modes: null block pointer");
  if (!E || !transl || !mode_sums || !status || !phase_l || !phase_r)
    return set_err(PF_ERR_ARG, "pf_modes: null pointer");
  if (max_iter <= 0 || nshift <= 0 || nshift > 2 * nl || nshift > 2 * nr)
    return set_err(PF_ERR_ARG, "pf_modes: bad max_iter or shift count");
  if (stride_l <= 0 || nl % stride_l != 0 || nrep_l <= 0 || nrep_l > stride_l || stride_r <= 0 ||
      nr % stride_r != 0 || nrep_r <= 0 || nrep_r > stride_r)
    return set_err(PF_ERR_ARG, "pf_modes: bad unfolding stride / representative count");
  if (!(a_z_l > 0.0) || !(a_z_r > 0.0) || !(lambda_eta > 0.0))
    return set_err(PF_ERR_ARG, "pf_modes: a_z and lambda_eta must be positive");
  if (npts == 0) return PF_SUCCESS;
  const MLayout lay = mlayout(n, nl, nr);
  const int S = (lay.m + 31) / 32;
  const int chunk = npts < kChunk ? npts : kChunk;
  const int grid = prep_grid(lay, chunk, S);
  if (grid <= 0) return set_err(PF_ERR_SIZE, "pf_modes: kernel does not fit on the device");
  if (!work || work_bytes < modes_bytes(lay, nq, chunk, grid))
    return set_err(PF_ERR_ARG, "pf_modes: workspace too small");
  MD_CUDA(cudaFuncSetAttribute(lead_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.task_smem));
  MD_CUDA(cudaFuncSetAttribute(tr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.task_smem));
  cudaStream_t st = (cudaStream_t)stream;
  int* queue = reinterpret_cast<int*>(work);
  const size_t mir = ((size_t)nq * 4 + 255) & ~(size_t)255;
  int* mirror = reinterpret_cast<int*>(reinterpret_cast<char*>(work) + 256);
  char* gscr = reinterpret_cast<char*>(work) + 256 + mir;
  Chunk ch;
  ch.base = gscr + (size_t)grid * lay.per_cta;
  ch.per_point = lay.per_point;
  ch.mat = lay.mat;
  pf::System<double> sys;
  sys.n = n;
  sys.nl = nl;
  sys.nr = nr;
  sys.L = L;
  sys.nq = nq;
  sys.HL = reinterpret_cast<const cx<double>*>(HL);
  sys.HLv = reinterpret_cast<const cx<double>*>(HLv);
  sys.HR = reinterpret_cast<const cx<double>*>(HR);
  sys.HRv = reinterpret_cast<const cx<double>*>(HRv);
  sys.Hd = reinterpret_cast<const cx<double>*>(Hd);
  sys.Hdv = reinterpret_cast<const cx<double>*>(Hdv);
  sys.Hld = reinterpret_cast<const cx<double>*>(Hld);
  sys.Hrd = reinterpret_cast<const cx<double>*>(Hrd);
  pf::Points pts{npts, E, qidx, zero_flag};
  pf::Params P{nullptr, eta, eta0, dev_factor, convergence, max_iter, 1};
  if (nl == nr) {
    mirror_kernel<<<nq, 256, 0, st>>>(HL, HLv, HR, HRv, 2 * nl * nl, nq, mirror);
    P.lead_mirror = mirror;
  }
  ModeGeom geo;
  geo.electron = (flags & PF_MODES_ELECTRON) != 0;
  geo.lambda_eta = lambda_eta;
  geo.a_z_l = a_z_l;
  geo.a_z_r = a_z_r;
  geo.nshift = nshift;
  geo.stride_l = stride_l;
  geo.nrep_l = nrep_l;
  geo.stride_r = stride_r;
  geo.nrep_r = nrep_r;
  geo.phase_l = reinterpret_cast<const cx<double>*>(phase_l);
  geo.phase_r = reinterpret_cast<const cx<double>*>(phase_r);
  ModeOut out{transl, transr, mode_sums, status, nprop, mode_kz, mode_bz, col_sums, nl > nr ? nl : nr, md2md};
  for (int p0 = 0; p0 < npts; p0 += chunk) {
    const int cnt = (npts - p0) < chunk ? (npts - p0) : chunk;
    MD_CUDA(cudaMemsetAsync(queue, 0, sizeof(int), st));
    const int g = grid < cnt ? grid : cnt;
    if (S == 1)
      prep_kernel<1><<<g, kPrepThreads, lay.prep_smem, st>>>(sys, pts, p0, cnt, P, lay, ch, gscr, queue, out);
    else
      prep_kernel<2><<<g, kPrepThreads, lay.prep_smem, st>>>(sys, pts, p0, cnt, P, lay, ch, gscr, queue, out);
    MD_CUDA(cudaGetLastError());
    lead_kernel<<<4 * cnt, kTaskThreads, lay.task_smem, st>>>(sys, pts, p0, cnt, lay, ch, geo, out);
    MD_CUDA(cudaGetLastError());
    tr_kernel<<<cnt, kTaskThreads, lay.task_smem, st>>>(sys, pts, p0, cnt, lay, ch, geo, eta, eta0, out);
    MD_CUDA(cudaGetLastError());
  }
  return PF_SUCCESS;
}

size_t pf_transport_tdb_blocks_workspace_size(int n, int nl, int nr, int nq, int npts) {
  return pf_transport_tdb_modes_workspace_size(n, nl, nr, nq, npts);
}

int pf_transport_tdb_blocks_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                                const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                                const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                                const int* zero_flag, double eta, double eta0, double dev_factor,
                                double convergence, int max_iter, double* transl, double* transr, int* status,
                                double* gl_adv, double* gl_plus, double* gr_ret, double* gr_minus, double* gml_adv,
                                double* gmr_ret, double* G_D_LR, double* G_R, double* G_D_RL, double* G_L,
                                void* work, size_t work_bytes, void* stream) {
  if (n <= 0 || nl <= 0 || nr <= 0 || L <= 0 || nq <= 0 || npts < 0)
    return set_err(PF_ERR_ARG, "pf_blocks: dimensions must be positive");
  if (n > PF_NMAX_RESIDENT || nl > PF_NMAX_RESIDENT || nr > PF_NMAX_RESIDENT)
    return set_err(PF_ERR_SIZE, "pf_blocks: block size exceeds the resident kernel limit");
  if (!HL || !HLv || !HR || !HRv || !Hd || !Hld || !Hrd || (L > 1 && !Hdv))
    return set_err(PF_ERR_ARG, "pf_blocks: null block pointer");
  if (!E || !transl || !status) return set_err(PF_ERR_ARG, "pf_blocks: null pointer");
  if (max_iter <= 0) return set_err(PF_ERR_ARG, "pf_blocks: bad max_iter");
  if (npts == 0) return PF_SUCCESS;
  const MLayout lay = mlayout(n, nl, nr);
  const int S = (lay.m + 31) / 32;
  const int chunk = npts < kChunk ? npts : kChunk;
  const int grid = prep_grid(lay, chunk, S);
  if (grid <= 0) return set_err(PF_ERR_SIZE, "pf_blocks: kernel does not fit on the device");
  if (!work || work_bytes < modes_bytes(lay, nq, chunk, grid))
    return set_err(PF_ERR_ARG, "pf_blocks: workspace too small");
  cudaStream_t st = (cudaStream_t)stream;
  int* queue = reinterpret_cast<int*>(work);
  const size_t mir = ((size_t)nq * 4 + 255) & ~(size_t)255;
  int* mirror = reinterpret_cast<int*>(reinterpret_cast<char*>(work) + 256);
  char* gscr = reinterpret_cast<char*>(work) + 256 + mir;
  Chunk ch;
  ch.base = gscr + (size_t)grid * lay.per_cta;
  ch.per_point = lay.per_point;
  ch.mat = lay.mat;
  pf::System<double> sys;
  sys.n = n;
  sys.nl = nl;
  sys.nr = nr;
  sys.L = L;
  sys.nq = nq;
  sys.HL = reinterpret_cast<const cx<double>*>(HL);
  sys.HLv = reinterpret_cast<const cx<double>*>(HLv);
  sys.HR = reinterpret_cast<const cx<double>*>(HR);
  sys.HRv = reinterpret_cast<const cx<double>*>(HRv);
  sys.Hd = reinterpret_cast<const cx<double>*>(Hd);
  sys.Hdv = reinterpret_cast<const cx<double>*>(Hdv);
  sys.Hld = reinterpret_cast<const cx<double>*>(Hld);
  sys.Hrd = reinterpret_cast<const cx<double>*>(Hrd);
  pf::Points pts{npts, E, qidx, zero_flag};
  pf::Params P{nullptr, eta, eta0, dev_factor, convergence, max_iter, 1};
  if (nl == nr) {
    mirror_kernel<<<nq, 256, 0, st>>>(HL, HLv, HR, HRv, 2 * nl * nl, nq, mirror);
    P.lead_mirror = mirror;
  }
  ModeOut out{transl, transr, nullptr, status, nullptr, nullptr, nullptr, nullptr, nl > nr ? nl : nr};
  BlockOut bo;
  double* const dst[NREC] = {gl_adv, gl_plus, gr_ret, gr_minus, gml_adv, gmr_ret, G_D_LR, G_R, G_D_RL, G_L};
  const int rows[NREC] = {nl, nl, nr, nr, nl, nr, nl, nr, nr, nl};
  const int cols[NREC] = {nl, nl, nr, nr, nl, nr, nr, nr, nl, nl};
  bool any = false;
  for (int k = 0; k < NREC; ++k) {
    bo.dst[k] = dst[k];
    bo.rows[k] = rows[k];
    bo.cols[k] = cols[k];
    any = any || dst[k] != nullptr;
  }
  for (int p0 = 0; p0 < npts; p0 += chunk) {
    const int cnt = (npts - p0) < chunk ? (npts - p0) : chunk;
    MD_CUDA(cudaMemsetAsync(queue, 0, sizeof(int), st));
    const int g = grid < cnt ? grid : cnt;
    if (S == 1)
      prep_kernel<1><<<g, kPrepThreads, lay.prep_smem, st>>>(sys, pts, p0, cnt, P, lay, ch, gscr, queue, out);
    else
      prep_kernel<2><<<g, kPrepThreads, lay.prep_smem, st>>>(sys, pts, p0, cnt, P, lay, ch, gscr, queue, out);
    MD_CUDA(cudaGetLastError());
    if (any) {
      blocks_out_kernel<<<dim3(cnt, NREC), 256, 0, st>>>(ch, p0, cnt, lay.ld, bo);
      MD_CUDA(cudaGetLastError());
    }
  }
  return PF_SUCCESS;
}

int pf_transport_tdb_modes_permode_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                                       const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                                       const double* Hld, const double* Hrd, int npts, const double* E,
                                       const int* qidx, const int* zero_flag, double eta, double eta0,
                                       double dev_factor, double convergence, int max_iter, double lambda_eta,
                                       double a_z_l, double a_z_r, int nshift, int stride_l, int nrep_l,
                                       const double* phase_l, int stride_r, int nrep_r, const double* phase_r,
                                       double* transl, double* transr, double* mode_sums, int* status, int* nprop,
                                       double* mode_kz, int* mode_bz, double* col_sums, void* work,
                                       size_t work_bytes, void* stream) {
  return pf_transport_tdb_modes_ex_dev(n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd, npts, E, qidx,
                                       zero_flag, eta, eta0, dev_factor, convergence, max_iter, lambda_eta, a_z_l,
                                       a_z_r, nshift, stride_l, nrep_l, phase_l, stride_r, nrep_r, phase_r, 0,
                                       transl, transr, mode_sums, status, nprop, mode_kz, mode_bz, col_sums, work,
                                       work_bytes, stream);
}

int pf_transport_tdb_modes_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                               const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                               const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                               const int* zero_flag, double eta, double eta0, double dev_factor, double convergence,
                               int max_iter, double lambda_eta, double a_z_l, double a_z_r, int nshift,
                               int stride_l, int nrep_l, const double* phase_l, int stride_r, int nrep_r,
                               const double* phase_r, double* transl, double* transr, double* mode_sums,
                               int* status, int* nprop, void* work, size_t work_bytes, void* stream) {
  return pf_transport_tdb_modes_permode_dev(n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd, npts, E, qidx,
                                            zero_flag, eta, eta0, dev_factor, convergence, max_iter, lambda_eta,
                                            a_z_l, a_z_r, nshift, stride_l, nrep_l, phase_l, stride_r, nrep_r,
                                            phase_r, transl, transr, mode_sums, status, nprop, nullptr, nullptr,
                                            nullptr, work, work_bytes, stream);
}

}  // extern "C"
