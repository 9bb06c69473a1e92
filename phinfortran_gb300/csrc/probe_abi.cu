// Buttiker probes of the tdb branch (buttiker = 1), one CTA per (omega, q)
// point, FP64:
//   * get_G_full_tdb with the probe self-energies (negf/lesser.f90:475-680):
//     the left-connected blocks GLeft_i (the last one closed with the right
//     lead, as the reference replaces it), the diagonal blocks G_full_i, the
//     couplings G_q_qp_i = G_{i,i+1}, and T_L;
//   * get_G_lesser_tdb (negf/lesser.f90:1199-1503): the left-connected and
//     full lesser functions, the probe fluxes, the lead fluxes and the
//     Jacobian d flux_i / d T_j of the temperature Newton iteration.
// The reference keeps every dGnL_i/dT_j (O(L^2) blocks a point); here the
// Jacobian is formed one probe j at a time: the seed dGnL_j/dT_j is carried
// to the right and then back through the full-lesser recursion, keeping
// O(L) blocks, with the same O(L^2 n^3) arithmetic.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "../../include/phinfortran_gb300.h"
#include "transport.cuh"

namespace {

using pf::cx;
using pf::Op;
using pf::opC;
using pf::opN;
using dcx = cx<double>;

thread_local char g_err[512] = "";
int set_err(int code, const char* msg) {
  snprintf(g_err, sizeof(g_err), "%s", msg);
  return code;
}
int cuda_err(cudaError_t e) {
  snprintf(g_err, sizeof(g_err), "pf_buttiker: %s", cudaGetErrorString(e));
  return PF_ERR_CUDA;
}

constexpr int kThreads = 256;

// C = base + acc
struct EpiBasePlus {
  dcx* c;
  int ld;
  Op<double> base;
  __device__ __forceinline__ void operator()(int r, int col, dcx acc) const {
    c[r + col * ld] = pf::cadd(base.at(r, col), acc);
  }
};
// C = base - acc
struct EpiBaseMinus {
  dcx* c;
  int ld;
  Op<double> base;
  __device__ __forceinline__ void operator()(int r, int col, dcx acc) const {
    c[r + col * ld] = pf::csub(base.at(r, col), acc);
  }
};
// C = acc + d I
struct EpiDiag {
  dcx* c;
  int ld;
  dcx d;
  __device__ __forceinline__ void operator()(int r, int col, dcx acc) const {
    c[r + col * ld] = (r == col) ? pf::cadd(acc, d) : acc;
  }
};

// CTA-wide complex sum reduction through red (>= 32 doubles); all threads
// get the result.
__device__ dcx block_sum(double re, double im, double* red) {
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) {
    red[2 * warp] = re;
    red[2 * warp + 1] = im;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    re = lane < nw ? red[2 * lane] : 0.0;
    im = lane < nw ? red[2 * lane + 1] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0) {
      red[0] = re;
      red[1] = im;
    }
  }
  __syncthreads();
  const dcx v = pf::mk<double>(red[0], red[1]);
  __syncthreads();
  return v;
}
// Tr(X) of an m x m matrix
__device__ dcx trace_c(const dcx* X, int ld, int m, double* red) {
  double re = 0.0, im = 0.0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    re += X[i + i * ld].x;
    im += X[i + i * ld].y;
  }
  return block_sum(re, im, red);
}
// Tr(X Y), X (m x n) and Y (n x m)
__device__ dcx trace_prod_c(const dcx* X, int ldx, Op<double> Y, int m, int n, double* red) {
  double re = 0.0, im = 0.0;
  for (int i = threadIdx.x; i < m * n; i += blockDim.x) {
    const int r = i % m, c = i / m;
    const dcx a = X[r + c * ldx];
    const dcx b = Y.at(c, r);
    re += a.x * b.x - a.y * b.y;
    im += a.x * b.y + a.y * b.x;
  }
  return block_sum(re, im, red);
}

struct PLayout {
  int m, ld, L;
  size_t mat, smem, per_cta;  // per_cta in complex elements
};

PLayout make_playout(int n, int nl, int nr, int L) {
  PLayout l;
  l.m = n > nl ? n : nl;
  l.m = l.m > nr ? l.m : nr;
  l.ld = l.m | 1;
  l.L = L;
  l.mat = (size_t)l.ld * l.m;
  l.smem = pf::NSM * l.mat * sizeof(dcx) + 32 * sizeof(double) + 2 * (size_t)l.m * sizeof(dcx) +
           (size_t)l.m * sizeof(int) + 64 * sizeof(int);
  // NG lead/work slots, GLeft, G_full, G_q_qp, GnL and one Jacobian column
  // (L each), plus BASE, Gamma_first, Gamma_last and an accumulator
  l.per_cta = ((size_t)pf::NG + 5 * (size_t)L + 4) * l.mat;
  return l;
}

struct ProbeIn {
  const double* sigw;   // [npts][L] complex probe self-energy
  const double* dsigw;  // [npts][L] complex d sigma / dT
  const double* f;      // [npts][L] Bose occupation at the probe temperatures
  const double* df;     // [npts][L] its temperature derivative
  const double* fL;     // [npts] left-lead occupation
  const double* fR;     // [npts] right-lead occupation
  const int* first;     // [npts] nonzero: the zero-frequency point (ie == 1)
};

struct ProbeOut {
  double* transl;      // [npts]
  double* flux_i;      // [npts][L] complex
  double* jac;         // [npts][L][L] complex, jac[p][i][j] = d flux_i / d T_j
  double* A_sum;       // [npts][L] complex Tr A_i
  double* Gn_i;        // [npts][L] complex Tr Gn_i
  double* flux_left;   // [npts] complex
  double* flux_right;  // [npts] complex
  int* status;         // [npts]
};

}  // namespace

namespace {

__device__ __forceinline__ dcx ld_c(const double* p, size_t i) { return pf::mk<double>(p[2 * i], p[2 * i + 1]); }
__device__ __forceinline__ void st_c(double* p, size_t i, dcx v) {
  p[2 * i] = v.x;
  p[2 * i + 1] = v.y;
}
__device__ __forceinline__ dcx cscale(dcx a, double s) { return pf::mk<double>(a.x * s, a.y * s); }

template <int S>
__global__ void __launch_bounds__(kThreads) probe_kernel(pf::System<double> sys, pf::Points pts, pf::Params P,
                                                         ProbeIn in, ProbeOut out, PLayout lay, dcx* gscr,
                                                         int* queue) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pf::Ctx<double> c;
  dcx* s = reinterpret_cast<dcx*>(smem_raw);
  for (int i = 0; i < pf::NSM; ++i) c.sm[i] = s + i * lay.mat;
  unsigned char* tail = reinterpret_cast<unsigned char*>(s + pf::NSM * lay.mat);
  c.red = reinterpret_cast<double*>(tail);
  c.iw.rowk = reinterpret_cast<dcx*>(tail + 32 * sizeof(double));
  c.iw.colk = c.iw.rowk + lay.m;
  int* ip = reinterpret_cast<int*>(c.iw.colk + lay.m);
  c.iw.perm = ip;
  c.iw.flag = ip + lay.m;
  c.ld = lay.ld;
  const size_t mat = lay.mat;
  const int L = sys.L, n = sys.n, nl = sys.nl, nr = sys.nr, ld = lay.ld;
  dcx* g0 = gscr + (size_t)blockIdx.x * lay.per_cta;
  for (int i = 0; i < pf::NG; ++i) c.gs[i] = g0 + i * mat;
  dcx* GLeft = g0 + pf::NG * mat;
  dcx* Gfull = GLeft + (size_t)L * mat;
  dcx* Gqqp = Gfull + (size_t)L * mat;
  dcx* GnL = Gqqp + (size_t)L * mat;
  dcx* dcol = GnL + (size_t)L * mat;
  dcx* BASE = dcol + (size_t)L * mat;
  dcx* GF = BASE + mat;
  dcx* GLAST = GF + mat;
  dcx* ACC = GLAST + mat;
  auto blk = [&](dcx* b, int i) { return b + (size_t)i * mat; };
  dcx* sm0 = c.sm[0];
  dcx* sm1 = c.sm[1];
  const Op<double> none = opN<double>(nullptr, 1);
  __shared__ int s_p;
  for (;;) {
    if (threadIdx.x == 0) s_p = atomicAdd(queue, 1);
    __syncthreads();
    const int p = s_p;
    __syncthreads();
    if (p >= pts.npts) break;
    const int q = pts.qidx ? pts.qidx[p] : 0;
    const double E = pts.E[p];
    const dcx* Hd = sys.Hd + (size_t)q * L * n * n;
    const dcx* Hdv = sys.Hdv + (size_t)q * (L - 1) * n * n;
    const dcx* Hld = sys.Hld + (size_t)q * nl * n;
    const dcx* Hrd = sys.Hrd + (size_t)q * nr * n;
    const dcx* HR = sys.HR + (size_t)q * nr * nr;
    int itl = 0, itr = 0;
    int st = pf::lead_pair<double, S>(c, sys, q, E, P, &itl, &itr);
    const double eps = E * P.eta + P.eta0;
    const dcx zD = pf::mk<double>(E, P.dev_factor * eps);
    const size_t pl = (size_t)p * L;
    // ---- left-to-right sweep with the probe self-energies; GLeft_i stored
    dcx* g = c.sm[3];
    dcx* A = c.sm[2];
    pf::copy_in(A, ld, opN<double>(c.gs[pf::G_GL], ld), nl, nl);
    pf::copy_in(sm0, ld, opN<double>(Hld, nl), nl, n);
    pf::row_gemm<double, S>(nl, n, nl, opN<double>(A, ld), opN<double>(sm0, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
    pf::row_gemm<double, S>(n, n, nl, opC<double>(sm0, ld), opN<double>(sm1, ld),
                        pf::EpiShift<double>{g, ld, pf::csub(zD, ld_c(in.sigw, pl)), opN<double>(Hd, n), true, none, false});
    st |= pf::inverse(g, ld, n, c.iw);
    pf::copy_out(blk(GLeft, 0), ld, false, g, ld, n, n);
    dcx* G0N = c.gs[pf::G_W2];
    dcx* U = c.gs[pf::G_W3];
    pf::row_gemm<double, S>(nl, n, n, opN<double>(sm1, ld), opN<double>(g, ld), pf::EpiStore<double>{G0N, ld, pf::mk<double>(1, 0)});
    for (int i = 1; i < L; ++i) {
      pf::copy_in(sm0, ld, opN<double>(Hdv + (size_t)(i - 1) * n * n, n), n, n);
      pf::row_gemm<double, S>(n, n, n, opN<double>(g, ld), opN<double>(sm0, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
      pf::row_gemm<double, S>(n, n, n, opC<double>(sm0, ld), opN<double>(sm1, ld),
                          pf::EpiShift<double>{A, ld, pf::csub(zD, ld_c(in.sigw, pl + i)),
                                               opN<double>(Hd + (size_t)i * n * n, n), true, none, false});
      if (i == L - 1) pf::copy_out(BASE, ld, false, A, ld, n, n);
      st |= pf::inverse(A, ld, n, c.iw);
      pf::copy_out(blk(GLeft, i), ld, false, A, ld, n, n);
      pf::row_gemm<double, S>(nl, n, n, opN<double>(G0N, ld), opN<double>(sm0, ld), pf::EpiStore<double>{U, ld, pf::mk<double>(1, 0)});
      pf::row_gemm<double, S>(nl, n, n, opN<double>(U, ld), opN<double>(A, ld), pf::EpiStore<double>{G0N, ld, pf::mk<double>(1, 0)});
      dcx* t = g;
      g = A;
      A = t;
    }
    // ---- right closure and Caroli T_L (g = last left-connected block)
    pf::copy_in(sm0, ld, opN<double>(Hrd, nr), nr, n);
    pf::row_gemm<double, S>(n, nr, n, opN<double>(g, ld), opC<double>(sm0, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
    pf::row_gemm<double, S>(nr, nr, n, opN<double>(sm0, ld), opN<double>(sm1, ld),
                        pf::EpiShift<double>{A, ld, zD, opN<double>(HR, nr), true, opN<double>(c.gs[pf::G_SR], ld), true});
    st |= pf::inverse(A, ld, nr, c.iw);
    pf::row_gemm<double, S>(nl, nr, n, opN<double>(G0N, ld), opC<double>(sm0, ld), pf::EpiStore<double>{U, ld, pf::mk<double>(1, 0)});
    pf::row_gemm<double, S>(nl, nr, nr, opN<double>(U, ld), opN<double>(A, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
    pf::copy_in(A, ld, opN<double>(c.gs[pf::G_GMR], ld), nr, nr);
    pf::row_gemm<double, S>(nl, nr, nr, opN<double>(sm1, ld), opN<double>(A, ld), pf::EpiStore<double>{U, ld, pf::mk<double>(1, 0)});
    pf::copy_in(A, ld, opN<double>(c.gs[pf::G_GML], ld), nl, nl);
    pf::row_gemm<double, S>(nr, nl, nl, opC<double>(sm1, ld), opN<double>(A, ld), pf::EpiStore<double>{g, ld, pf::mk<double>(1, 0)});
    const double tl = pf::trace_prod_re(U, ld, opN<double>(g, ld), nl, nr, c.red);
    // ---- GLeft_{L-1} <- inv(BASE - Hrd^H gr Hrd) (Gblock_NN1); G_full_{L-1} = the same
    dcx* X = c.sm[2];
    dcx* Y = c.sm[3];
    pf::copy_in(sm0, ld, opN<double>(c.gs[pf::G_GR], ld), nr, nr);
    pf::row_gemm<double, S>(n, nr, nr, opC<double>(Hrd, nr), opN<double>(sm0, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
    pf::copy_in(sm0, ld, opN<double>(Hrd, nr), nr, n);
    pf::row_gemm<double, S>(n, n, nr, opN<double>(sm1, ld), opN<double>(sm0, ld), EpiBaseMinus{X, ld, opN<double>(BASE, ld)});
    st |= pf::inverse(X, ld, n, c.iw);
    pf::copy_out(blk(GLeft, L - 1), ld, false, X, ld, n, n);
    pf::copy_out(blk(Gfull, L - 1), ld, false, X, ld, n, n);
    // ---- G_q_qp_i = GLeft_i V G_full_{i+1}; G_full_i = GLeft_i + G_q_qp_i V^H GLeft_i
    dcx* Gnext = X;
    dcx* other = Y;
    for (int i = L - 2; i >= 0; --i) {
      pf::copy_in(sm0, ld, opN<double>(Hdv + (size_t)i * n * n, n), n, n);
      pf::row_gemm<double, S>(n, n, n, opN<double>(blk(GLeft, i), ld), opN<double>(sm0, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
      pf::row_gemm<double, S>(n, n, n, opN<double>(sm1, ld), opN<double>(Gnext, ld), pf::EpiStore<double>{other, ld, pf::mk<double>(1, 0)});
      pf::copy_out(blk(Gqqp, i), ld, false, other, ld, n, n);
      pf::row_gemm<double, S>(n, n, n, opN<double>(other, ld), opC<double>(sm0, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
      pf::copy_in(Gnext, ld, opN<double>(blk(GLeft, i), ld), n, n);
      pf::row_gemm<double, S>(n, n, n, opN<double>(sm1, ld), opN<double>(Gnext, ld), EpiBasePlus{other, ld, opN<double>(Gnext, ld)});
      pf::copy_out(blk(Gfull, i), ld, false, other, ld, n, n);
      dcx* t = Gnext;
      Gnext = other;
      other = t;
    }
    // ---- lead escape rates Gamma_first = i(S - S^H), S = Hld^H gl Hld; Gamma_last likewise
    pf::copy_in(sm0, ld, opN<double>(Hld, nl), nl, n);
    pf::copy_in(X, ld, opN<double>(c.gs[pf::G_GL], ld), nl, nl);
    pf::row_gemm<double, S>(nl, n, nl, opN<double>(X, ld), opN<double>(sm0, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
    pf::row_gemm<double, S>(n, n, nl, opC<double>(sm0, ld), opN<double>(sm1, ld), pf::EpiStore<double>{Y, ld, pf::mk<double>(1, 0)});
    pf::gamma_from_sigma(GF, ld, Y, ld, n, +1);
    pf::copy_in(sm0, ld, opN<double>(Hrd, nr), nr, n);
    pf::copy_in(X, ld, opN<double>(c.gs[pf::G_GR], ld), nr, nr);
    pf::row_gemm<double, S>(nr, n, nr, opN<double>(X, ld), opN<double>(sm0, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
    pf::row_gemm<double, S>(n, n, nr, opC<double>(sm0, ld), opN<double>(sm1, ld), pf::EpiStore<double>{Y, ld, pf::mk<double>(1, 0)});
    pf::gamma_from_sigma(GLAST, ld, Y, ld, n, +1);
    // ---- per-layer scalars
    const double freq = sqrt(E);
    const bool first = in.first && in.first[p];
    const double fL = in.fL[p], fR = in.fR[p];
    // probe escape rates gamma_i = i (sigma - conj sigma) (a multiple of I)
    auto gam = [&](const double* sv, int i) {
      const dcx sg = ld_c(sv, pl + i);
      return pf::mk<double>(-2.0 * sg.y, 0.0);
    };
    // ---- spectral traces Tr A_i = -2 Im Tr G_full_i
    // flux_left = Tr(Gamma_first A_0) fL
    //   Tr(G A) = i Tr(G F) - i Tr(G F^H) for A = i (F - F^H)
    auto tr_gamma_A = [&](const dcx* Gam, const dcx* F) {
      const dcx t1 = trace_prod_c(Gam, ld, opN<double>(F, ld), n, n, c.red);
      const dcx t2 = trace_prod_c(Gam, ld, opC<double>(F, ld), n, n, c.red);
      const dcx d = pf::csub(t1, t2);
      return pf::mk<double>(-d.y, d.x);   // i (t1 - t2)
    };
    dcx fluxl = cscale(tr_gamma_A(GF, blk(Gfull, 0)), fL);
    dcx fluxr = cscale(tr_gamma_A(GLAST, blk(Gfull, L - 1)), fR);
    // ---- left-connected lesser function, left to right
    for (int i = 0; i < L; ++i) {
      const dcx gi = gam(in.sigw, i);
      const dcx di = cscale(gi, in.f[pl + i]);
      if (i == 0) {
        // sigma_in = Gamma_first fL + gamma_0 f_0 I
        for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
          const int r = t % n, col = t / n;
          dcx v = cscale(GF[r + col * ld], fL);
          if (r == col) v = pf::cadd(v, di);
          sm1[r + col * ld] = v;
        }
        __syncthreads();
      } else {
        pf::copy_in(sm0, ld, opN<double>(Hdv + (size_t)(i - 1) * n * n, n), n, n);
        pf::row_gemm<double, S>(n, n, n, opN<double>(blk(GnL, i - 1), ld), opN<double>(sm0, ld),
                            pf::EpiStore<double>{X, ld, pf::mk<double>(1, 0)});
        pf::row_gemm<double, S>(n, n, n, opC<double>(sm0, ld), opN<double>(X, ld), EpiDiag{sm1, ld, di});
        if (i == L - 1) {
          for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
            const int r = t % n, col = t / n;
            sm1[r + col * ld] = pf::cadd(sm1[r + col * ld], cscale(GLAST[r + col * ld], fR));
          }
          __syncthreads();
        }
      }
      pf::row_gemm<double, S>(n, n, n, opN<double>(blk(GLeft, i), ld), opN<double>(sm1, ld),
                          pf::EpiStore<double>{X, ld, pf::mk<double>(1, 0)});
      pf::row_gemm<double, S>(n, n, n, opN<double>(X, ld), opC<double>(blk(GLeft, i), ld),
                          pf::EpiStore<double>{blk(GnL, i), ld, pf::mk<double>(1, 0)});
    }
    // ---- full lesser function, right to left: Gn_i = GnL_i + G V Gn_{i+1} V^H G^H + GnL V Q^H + Q V^H GnL
    // (one step; src = Gn_{i+1} in shared memory Y, result into Y; `seed` null for the
    // Jacobian rows left of the probe where dGnL vanishes)
    auto back_step = [&](int i, const dcx* seed) {
      pf::copy_in(sm0, ld, opN<double>(Hdv + (size_t)i * n * n, n), n, n);
      pf::row_gemm<double, S>(n, n, n, opN<double>(sm0, ld), opN<double>(Y, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
      pf::row_gemm<double, S>(n, n, n, opN<double>(sm1, ld), opC<double>(sm0, ld), pf::EpiStore<double>{X, ld, pf::mk<double>(1, 0)});
      pf::row_gemm<double, S>(n, n, n, opN<double>(blk(GLeft, i), ld), opN<double>(X, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
      if (seed) {
        pf::row_gemm<double, S>(n, n, n, opN<double>(sm1, ld), opC<double>(blk(GLeft, i), ld),
                            EpiBasePlus{ACC, ld, opN<double>(seed, ld)});
        pf::row_gemm<double, S>(n, n, n, opN<double>(seed, ld), opN<double>(sm0, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
        pf::row_gemm<double, S>(n, n, n, opN<double>(sm1, ld), opC<double>(blk(Gqqp, i), ld), pf::EpiAcc<double>{ACC, ld});
        pf::row_gemm<double, S>(n, n, n, opN<double>(blk(Gqqp, i), ld), opC<double>(sm0, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
        pf::copy_in(X, ld, opN<double>(seed, ld), n, n);
        pf::row_gemm<double, S>(n, n, n, opN<double>(sm1, ld), opN<double>(X, ld), pf::EpiAcc<double>{ACC, ld});
      } else {
        pf::row_gemm<double, S>(n, n, n, opN<double>(sm1, ld), opC<double>(blk(GLeft, i), ld),
                            pf::EpiStore<double>{ACC, ld, pf::mk<double>(1, 0)});
      }
      pf::copy_in(Y, ld, opN<double>(ACC, ld), n, n);
    };
    pf::copy_in(Y, ld, opN<double>(blk(GnL, L - 1), ld), n, n);
    dcx trGn_last = trace_c(Y, ld, n, c.red);
    fluxr = cscale(pf::csub(fluxr, trace_prod_c(GLAST, ld, opN<double>(Y, ld), n, n, c.red)), freq);
    for (int i = L - 1; i >= 0; --i) {
      if (i < L - 1) back_step(i, blk(GnL, i));
      const dcx trGn = (i == L - 1) ? trGn_last : trace_c(Y, ld, n, c.red);
      const dcx trG = trace_c(blk(Gfull, i), ld, n, c.red);
      const dcx trA = first ? pf::mk<double>(0, 0) : pf::mk<double>(-2.0 * trG.y, 0.0);
      const dcx tGn = first ? pf::mk<double>(0, 0) : trGn;
      const dcx gi = gam(in.sigw, i);
      if (i == 0) fluxl = cscale(pf::csub(fluxl, trace_prod_c(GF, ld, opN<double>(Y, ld), n, n, c.red)), freq);
      if (threadIdx.x == 0) {
        // flux_i = -Tr(gamma_i Gn_i) + Tr(gamma_i A_i) f_i
        const dcx fl = pf::cadd(pf::mk<double>(-(gi.x * tGn.x - gi.y * tGn.y), -(gi.x * tGn.y + gi.y * tGn.x)),
                                cscale(pf::cmul(gi, trA), in.f[pl + i]));
        st_c(out.flux_i, pl + i, fl);
        st_c(out.A_sum, pl + i, trA);
        st_c(out.Gn_i, pl + i, tGn);
      }
    }
    // ---- Jacobian, one probe temperature T_j at a time:
    //   dGnL_j/dT_j = GLeft_j c_j GLeft_j^H, c_j = gamma_j df_j + dgamma_j f_j
    //   dGnL_i/dT_j = GLeft_i V^H dGnL_{i-1} V GLeft_i^H   (i > j), 0 for i < j
    //   dGn_i/dT_j  by the full-lesser recursion; jac(i, j) = -gamma_i Tr dGn_i/dT_j
    //   (+ the explicit term on i == j)
    const size_t pjj = (size_t)p * L * L;
    for (int j = 0; j < L; ++j) {
      const dcx gj = gam(in.sigw, j), dgj = gam(in.dsigw, j);
      const dcx cj = pf::cadd(cscale(gj, in.df[pl + j]), cscale(dgj, in.f[pl + j]));
      pf::row_gemm<double, S>(n, n, n, opN<double>(blk(GLeft, j), ld), opC<double>(blk(GLeft, j), ld),
                          pf::EpiStore<double>{blk(dcol, j), ld, cj});
      for (int i = j + 1; i < L; ++i) {
        pf::copy_in(sm0, ld, opN<double>(Hdv + (size_t)(i - 1) * n * n, n), n, n);
        pf::row_gemm<double, S>(n, n, n, opN<double>(blk(dcol, i - 1), ld), opN<double>(sm0, ld),
                            pf::EpiStore<double>{X, ld, pf::mk<double>(1, 0)});
        pf::row_gemm<double, S>(n, n, n, opC<double>(sm0, ld), opN<double>(X, ld), pf::EpiStore<double>{sm1, ld, pf::mk<double>(1, 0)});
        pf::row_gemm<double, S>(n, n, n, opN<double>(blk(GLeft, i), ld), opN<double>(sm1, ld),
                            pf::EpiStore<double>{X, ld, pf::mk<double>(1, 0)});
        pf::row_gemm<double, S>(n, n, n, opN<double>(X, ld), opC<double>(blk(GLeft, i), ld),
                            pf::EpiStore<double>{blk(dcol, i), ld, pf::mk<double>(1, 0)});
      }
      pf::copy_in(Y, ld, opN<double>(blk(dcol, L - 1), ld), n, n);
      for (int i = L - 1; i >= 0; --i) {
        if (i < L - 1) back_step(i, i >= j ? blk(dcol, i) : nullptr);
        const dcx tr = trace_c(Y, ld, n, c.red);
        const dcx gi = gam(in.sigw, i);
        dcx v = pf::mk<double>(-(gi.x * tr.x - gi.y * tr.y), -(gi.x * tr.y + gi.y * tr.x));
        if (i == j) {
          const dcx trG = trace_c(blk(Gfull, i), ld, n, c.red);
          const dcx trA = pf::mk<double>(-2.0 * trG.y, 0.0);
          const dcx dgi = gam(in.dsigw, i);
          v = pf::cadd(v, pf::cadd(cscale(pf::cmul(gi, trA), in.df[pl + j]), cscale(pf::cmul(dgi, trA), in.f[pl + j])));
        }
        if (threadIdx.x == 0) st_c(out.jac, pjj + (size_t)i * L + j, first ? pf::mk<double>(0, 0) : v);
      }
    }
    if (threadIdx.x == 0) {
      const bool zero = pts.zero_flag && pts.zero_flag[p];
      double a = tl;
      if (zero || a < 1.0e-60) a = 0.0;
      out.transl[p] = a;
      st_c(out.flux_left, p, fluxl);
      st_c(out.flux_right, p, fluxr);
      out.status[p] = st;
    }
    __syncthreads();
  }
}

}  // namespace

namespace {

struct DevMem {
  std::vector<void*> ptrs;
  ~DevMem() {
    for (void* p : ptrs) cudaFree(p);
  }
  cudaError_t alloc(void** d, size_t bytes) {
    cudaError_t e = cudaMalloc(d, bytes ? bytes : 1);
    if (e == cudaSuccess) ptrs.push_back(*d);
    return e;
  }
  template <typename T>
  cudaError_t up(T** d, const T* h, size_t n) {
    cudaError_t e = alloc((void**)d, n * sizeof(T));
    if (e != cudaSuccess || n == 0 || !h) return e;
    return cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice);
  }
};

template <int S>
int probe_grid(const PLayout& lay, int npts) {
  auto k = probe_kernel<S>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.smem) != cudaSuccess) return -1;
  int per_sm = 0, dev = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, lay.smem) != cudaSuccess || per_sm < 1)
    return -1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int g = sms * per_sm;
  return g < npts ? g : npts;
}

}  // namespace

extern "C" {

const char* pf_buttiker_last_error(void) { return g_err; }

int pf_buttiker_tdb(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv, const double* HR,
                    const double* HRv, const double* Hd, const double* Hdv, const double* Hld, const double* Hrd,
                    int npts, const double* E, const int* qidx, const int* first, const double* sigw,
                    const double* dsigw, const double* f, const double* df, const double* fL, const double* fR,
                    double eta, double eta0, double dev_factor, double convergence, int max_iter, double* transl,
                    double* flux_i, double* jac, double* A_sum, double* Gn_i, double* flux_left,
                    double* flux_right, int* status) {
  if (n <= 0 || nl <= 0 || nr <= 0 || nq <= 0 || npts < 0) return set_err(PF_ERR_ARG, "pf_buttiker: bad sizes");
  if (L < 2) return set_err(PF_ERR_ARG, "pf_buttiker: the probe recursion needs at least two device layers");
  if (n > PF_NMAX_RESIDENT || nl > PF_NMAX_RESIDENT || nr > PF_NMAX_RESIDENT)
    return set_err(PF_ERR_SIZE, "pf_buttiker: block size above the resident limit");
  if (max_iter <= 0) return set_err(PF_ERR_ARG, "pf_buttiker: max_iter must be positive");
  if (npts == 0) return PF_SUCCESS;
  if (!HL || !HLv || !HR || !HRv || !Hd || !Hdv || !Hld || !Hrd || !E || !sigw || !dsigw || !f || !df || !fL ||
      !fR || !transl || !flux_i || !jac || !A_sum || !Gn_i || !flux_left || !flux_right || !status)
    return set_err(PF_ERR_ARG, "pf_buttiker: null pointer");
  if (qidx)
    for (int p = 0; p < npts; ++p)
      if (qidx[p] < 0 || qidx[p] >= nq) return set_err(PF_ERR_ARG, "pf_buttiker: qidx out of range");
  const PLayout lay = make_playout(n, nl, nr, L);
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (lay.smem > (size_t)optin) return set_err(PF_ERR_SIZE, "pf_buttiker: working set exceeds shared memory");
  const int S = (lay.m + 31) / 32;
  const int grid = (S == 1) ? probe_grid<1>(lay, npts) : probe_grid<2>(lay, npts);
  if (grid <= 0) return set_err(PF_ERR_SIZE, "pf_buttiker: kernel does not fit on the device");
  // identical leads (bitwise) reuse the left decimation, as the transport entries do
  std::vector<int> mirror(nq, 0);
  if (nl == nr)
    for (int q = 0; q < nq; ++q) {
      const size_t off = 2 * (size_t)q * nl * nl, cnt = 2 * (size_t)nl * nl;
      mirror[q] = memcmp(HL + off, HR + off, cnt * 8) == 0 && memcmp(HLv + off, HRv + off, cnt * 8) == 0;
    }
  DevMem d;
  double *dHL, *dHLv, *dHR, *dHRv, *dHd, *dHdv, *dHld, *dHrd, *dE, *dsw, *ddsw, *df_, *ddf, *dfL, *dfR;
  int *dq = nullptr, *dfirst = nullptr, *dmir, *queue;
  cudaError_t e;
  const size_t nn = 2 * (size_t)n * n;
  if ((e = d.up(&dHL, HL, 2 * (size_t)nq * nl * nl)) != cudaSuccess ||
      (e = d.up(&dHLv, HLv, 2 * (size_t)nq * nl * nl)) != cudaSuccess ||
      (e = d.up(&dHR, HR, 2 * (size_t)nq * nr * nr)) != cudaSuccess ||
      (e = d.up(&dHRv, HRv, 2 * (size_t)nq * nr * nr)) != cudaSuccess ||
      (e = d.up(&dHd, Hd, (size_t)nq * L * nn)) != cudaSuccess ||
      (e = d.up(&dHdv, Hdv, (size_t)nq * (L - 1) * nn)) != cudaSuccess ||
      (e = d.up(&dHld, Hld, 2 * (size_t)nq * nl * n)) != cudaSuccess ||
      (e = d.up(&dHrd, Hrd, 2 * (size_t)nq * nr * n)) != cudaSuccess ||
      (e = d.up(&dE, E, (size_t)npts)) != cudaSuccess ||
      (e = d.up(&dsw, sigw, 2 * (size_t)npts * L)) != cudaSuccess ||
      (e = d.up(&ddsw, dsigw, 2 * (size_t)npts * L)) != cudaSuccess ||
      (e = d.up(&df_, f, (size_t)npts * L)) != cudaSuccess ||
      (e = d.up(&ddf, df, (size_t)npts * L)) != cudaSuccess ||
      (e = d.up(&dfL, fL, (size_t)npts)) != cudaSuccess ||
      (e = d.up(&dfR, fR, (size_t)npts)) != cudaSuccess ||
      (e = d.up(&dmir, mirror.data(), mirror.size())) != cudaSuccess ||
      (qidx && (e = d.up(&dq, qidx, (size_t)npts)) != cudaSuccess) ||
      (first && (e = d.up(&dfirst, first, (size_t)npts)) != cudaSuccess) ||
      (e = d.alloc((void**)&queue, sizeof(int))) != cudaSuccess)
    return cuda_err(e);
  double *oT, *oflux, *ojac, *oA, *oGn, *ofl, *ofr;
  int* ost;
  dcx* gscr;
  if ((e = d.alloc((void**)&oT, 8 * (size_t)npts)) != cudaSuccess ||
      (e = d.alloc((void**)&oflux, 16 * (size_t)npts * L)) != cudaSuccess ||
      (e = d.alloc((void**)&ojac, 16 * (size_t)npts * L * L)) != cudaSuccess ||
      (e = d.alloc((void**)&oA, 16 * (size_t)npts * L)) != cudaSuccess ||
      (e = d.alloc((void**)&oGn, 16 * (size_t)npts * L)) != cudaSuccess ||
      (e = d.alloc((void**)&ofl, 16 * (size_t)npts)) != cudaSuccess ||
      (e = d.alloc((void**)&ofr, 16 * (size_t)npts)) != cudaSuccess ||
      (e = d.alloc((void**)&ost, 4 * (size_t)npts)) != cudaSuccess ||
      (e = d.alloc((void**)&gscr, (size_t)grid * lay.per_cta * sizeof(dcx))) != cudaSuccess ||
      (e = cudaMemset(queue, 0, sizeof(int))) != cudaSuccess)
    return cuda_err(e);
  pf::System<double> sys;
  sys.n = n;
  sys.nl = nl;
  sys.nr = nr;
  sys.L = L;
  sys.nq = nq;
  sys.HL = reinterpret_cast<const dcx*>(dHL);
  sys.HLv = reinterpret_cast<const dcx*>(dHLv);
  sys.HR = reinterpret_cast<const dcx*>(dHR);
  sys.HRv = reinterpret_cast<const dcx*>(dHRv);
  sys.Hd = reinterpret_cast<const dcx*>(dHd);
  sys.Hdv = reinterpret_cast<const dcx*>(dHdv);
  sys.Hld = reinterpret_cast<const dcx*>(dHld);
  sys.Hrd = reinterpret_cast<const dcx*>(dHrd);
  pf::Points pts{npts, dE, dq, dfirst};
  pf::Params P{dmir, eta, eta0, dev_factor, convergence, max_iter, 0};
  ProbeIn in{dsw, ddsw, df_, ddf, dfL, dfR, dfirst};
  ProbeOut out{oT, oflux, ojac, oA, oGn, ofl, ofr, ost};
  if (S == 1)
    probe_kernel<1><<<grid, kThreads, lay.smem>>>(sys, pts, P, in, out, lay, gscr, queue);
  else
    probe_kernel<2><<<grid, kThreads, lay.smem>>>(sys, pts, P, in, out, lay, gscr, queue);
  if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaDeviceSynchronize()) != cudaSuccess) return cuda_err(e);
  if ((e = cudaMemcpy(transl, oT, 8 * (size_t)npts, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(flux_i, oflux, 16 * (size_t)npts * L, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(jac, ojac, 16 * (size_t)npts * L * L, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(A_sum, oA, 16 * (size_t)npts * L, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(Gn_i, oGn, 16 * (size_t)npts * L, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(flux_left, ofl, 16 * (size_t)npts, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(flux_right, ofr, 16 * (size_t)npts, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(status, ost, 4 * (size_t)npts, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda_err(e);
  for (int p = 0; p < npts; ++p)
    if (status[p]) return set_err(PF_ERR_POINT, "pf_buttiker: a point reported a singular or non-finite block");
  return PF_SUCCESS;
}

}  // extern "C"
