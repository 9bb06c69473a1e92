// extern "C" entry of the large-block transport path (block sizes above the
// shared-memory resident kernels: the diamond slabs with n = 96..384 DOF
// per layer, the 3-orbital ribbons with n = 768).
//
// Points are grouped by q (their blocks are then shared operands) and run
// in batches that advance together: the Lopez-Sancho decimations of the
// two leads (surface.f90:479-568) with a per-point convergence mask, the
// left-to-right RGF sweep (lesser.f90:547-654) and the Caroli trace
// (lesser.f90:787-800).  Every step is one launch over the batch (tiled.cuh);
// the host only drives the loop and reads one counter per decimation step.
#include <cuda_runtime.h>
#include <stdio.h>

#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

#include "../../include/phinfortran_gb300.h"
#include "tc_gemm.h"
#include "tiled.cuh"
#include "transport.cuh"

using pf::cx;
using namespace pf::tiled;

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
#define TL_CUDA(call)                                  \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_err(e_, #call); \
  } while (0)

constexpr int kMaxBatch = 256;
constexpr size_t kBatchBytes = (size_t)6 << 30;
// Tuning set by pf_tiled_set_tuning (0: the built-in choice): the panel
// width of the blocked Gauss-Jordan inverse and the most points a batch.
int g_tune_panel = 0;
int g_tune_batch = 0;
constexpr size_t kSmallInvBytes = 200 * 1024;
constexpr size_t kPanelBytes = 200 * 1024;
constexpr int kMats = 16;  // per-point working matrices

// complex constant for host code (pf::mk and df64(int) are device-only)
template <typename T>
__host__ __device__ inline cx<T> hmk(T a, T b) {
  cx<T> z;
  z.x = a;
  z.y = b;
  return z;
}
template <typename T>
inline T hval(double v);
template <>
inline double hval<double>(double v) {
  return v;
}
template <>
inline pf::df64 hval<pf::df64>(double v) {  // exact for the constants used here (0, 1, -1)
  return pf::df64((float)v, 0.f);
}
template <typename T>
inline cx<T> hc(double re) {
  return hmk<T>(hval<T>(re), hval<T>(0.0));
}

__global__ void k_to_df64(const double* __restrict__ src, pf::df64* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = pf::df64(src[i]);
}

// ---------------------------------------------------------------------------
// elementwise kernels (grid: (ceil(m*m/256), batch))
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_shift_neg(cx<T>* dst, const cx<T>* src, long long stride, int m, int ld, const cx<T>* z,
                            const int* active) {
  const int b = blockIdx.y;
  if (active && !active[b]) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m * m) return;
  const int r = i % m, c = i / m;
  cx<T> v = src[(size_t)b * stride + r + (size_t)c * ld];
  v = pf::mk<T>(-v.x, -v.y);
  if (r == c) v = pf::cadd(v, z[b]);
  dst[(size_t)b * stride + r + (size_t)c * ld] = v;
}
// dst_b = op(src) with src shared (stride 0) or per point; conj_t: conjugate transpose
template <typename T>
__global__ void k_copy(cx<T>* dst, long long sd, const cx<T>* src, long long ss, int lds, int rows, int cols,
                       int ldd, int conj_t) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  const int r = i % rows, c = i / rows;
  const cx<T> v =
      conj_t ? pf::cconj(src[(size_t)b * ss + c + (size_t)r * lds]) : src[(size_t)b * ss + r + (size_t)c * lds];
  dst[(size_t)b * sd + r + (size_t)c * ldd] = v;
}
template <typename T>
__global__ void k_add2(cx<T>* a, cx<T>* b2, const cx<T>* t, long long stride, int m, int ld, const int* active) {
  const int b = blockIdx.y;
  if (active && !active[b]) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m * m) return;
  const size_t o = (size_t)b * stride + (i % m) + (size_t)(i / m) * ld;
  a[o] = pf::cadd(a[o], t[o]);
  b2[o] = pf::cadd(b2[o], t[o]);
}
template <typename T>
__global__ void k_sub(cx<T>* a, const cx<T>* s, long long stride, int m, int ld) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m * m) return;
  const size_t o = (size_t)b * stride + (i % m) + (size_t)(i / m) * ld;
  a[o] = pf::csub(a[o], s[o]);
}
// G = sgn * i (S - S^H), sgn = +1 or -1
template <typename T>
__global__ void k_gamma(cx<T>* G, const cx<T>* S, long long stride, int m, int ld, int sgn) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m * m) return;
  const int r = i % m, c = i / m;
  const cx<T> a = S[(size_t)b * stride + r + (size_t)c * ld];
  const cx<T> e = S[(size_t)b * stride + c + (size_t)r * ld];
  const cx<T> d = pf::mk<T>(a.x - e.x, a.y + e.y);  // a - conj(e)
  G[(size_t)b * stride + r + (size_t)c * ld] = sgn > 0 ? pf::mk<T>(-d.y, d.x) : pf::mk<T>(d.y, -d.x);
}
// per-point energies: zl = E - i eps, zr = E + i eps, zd = E + i dev eps
template <typename T>
__global__ void k_points(const double* E, const int* idx, int cnt, double eta, double eta0, double devf,
                         cx<T>* zl, cx<T>* zr, cx<T>* zd, int* st) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= cnt) return;
  const double e = E[idx[b]];
  const double eps = e * eta + eta0;
  zl[b] = pf::mk<T>(T(e), T(-eps));
  zr[b] = pf::mk<T>(T(e), T(eps));
  zd[b] = pf::mk<T>(T(e), T(devf * eps));
  st[b] = 0;
}
__global__ void k_fill(int* a, int n, int v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}
__global__ void k_iota(int* a, int n, int start) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = start + i;
}
// decimation control: maxdiff of alpha per point, retire converged points
template <typename T>
__global__ void k_converge(const cx<T>* al, long long stride, int m, int ld, double conv, int max_iter, int* active,
                           int* it, int* st, int* count, int first) {
  const int b = blockIdx.x;
  if (!active[b]) return;
  double v = 0.0;
  for (int i = threadIdx.x; i < m * m; i += blockDim.x) {
    const cx<T> e = al[(size_t)b * stride + (i % m) + (size_t)(i / m) * ld];
    const double h = hypot(pf::to_d(e.x), pf::to_d(e.y));
    v = (h > v || h != h) ? h : v;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w > v || w != w) ? w : v;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    v = red[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = (red[w] > v || red[w] != red[w]) ? red[w] : v;
    if (!first) it[b] += 1;
    if (v != v) {
      st[b] |= pf::PF_NAN;
      active[b] = 0;
    } else if (!(v > conv)) {
      active[b] = 0;
    } else if (it[b] >= max_iter) {
      st[b] |= pf::PF_NOT_CONVERGED;
      active[b] = 0;
    } else {
      atomicAdd(count, 1);
    }
  }
}
// T = Re Tr(P Q), P (m x k), Q (k x m); scatter to the point's slot
template <typename T>
__global__ void k_trace(const cx<T>* P, const cx<T>* Q, long long stride, int m, int k, int ld, const int* idx,
                        const int* zero_flag, const int* st, const int* itl, const int* itr, double* transl,
                        int* status, int* iters) {
  const int b = blockIdx.x;
  double v = 0.0;
  for (int i = threadIdx.x; i < m * k; i += blockDim.x) {
    const int r = i % m, c = i / m;
    const cx<T> a = P[(size_t)b * stride + r + (size_t)c * ld];
    const cx<T> q = Q[(size_t)b * stride + c + (size_t)r * ld];
    v += pf::to_d(a.x) * pf::to_d(q.x) - pf::to_d(a.y) * pf::to_d(q.y);
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w];
    const int p = idx[b];
    const bool zero = zero_flag && zero_flag[p];
    transl[p] = (zero || v < 1.0e-60) ? 0.0 : v;
    status[p] = st[b];
    if (iters) {
      iters[2 * p] = itl[b];
      iters[2 * p + 1] = itr[b];
    }
  }
}
__global__ void k_mirror(const double* HL, const double* HLv, const double* HR, const double* HRv, size_t m2,
                         int* diff) {
  int d = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < m2; i += (size_t)gridDim.x * blockDim.x)
    d |= (__double_as_longlong(HL[i]) != __double_as_longlong(HR[i])) |
         (__double_as_longlong(HLv[i]) != __double_as_longlong(HRv[i]));
  if (d) atomicOr(diff, 1);
}

// ---------------------------------------------------------------------------
// block-circulant leads (circular_flag = 1, negf/circular.f90:42-105)
//
// A lead of ny x nx Bloch cells has block-circulant matrices: ny outer
// blocks of na = m / ny rows, each of them nx inner blocks of s = na / nx.
// The two-level Fourier transform of their first block rows
// (util.f90:732-756, applied along y then along x) makes them block
// diagonal; each of the K = ny nx small s x s blocks is decimated on its own
// (util.f90:761-799) and the result transformed back with the unitary
// P1 = F_y (x) 1, P2 = F_x (x) 1 of set_pmatrix (circular.f90:9-38).
// ---------------------------------------------------------------------------
// dst_b = op(src_{b mod period}) (src stride ss; ss = 0: one shared source)
template <typename T>
__global__ void k_copy_per(cx<T>* dst, long long sd, const cx<T>* src, long long ss, int period, int lds, int rows,
                           int cols, int ldd, int conj_t) {
  const int b = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  const int r = i % rows, c = i / rows;
  const cx<T>* sp = src + (size_t)(b % period) * ss;
  const cx<T> v = conj_t ? pf::cconj(sp[c + (size_t)r * lds]) : sp[r + (size_t)c * lds];
  dst[(size_t)b * sd + r + (size_t)c * ldd] = v;
}
// Small block kb = i nx + j (s x s, ld s) of the lead's transforms:
//   hs[kb](r, c) = sum_l w_x^{j l} sum_p w_y^{i p} h00(r, p na + l s + c)
// (w_y = exp(i gry / ny), w_x = exp(i grx / nx)); the same of alpha = v^H,
// stored conjugate-transposed (vs[kb] = alpha_s[kb]^H), the form decimate()
// takes its coupling in (alpha0 = v^H, beta0 = v; util.f90 decimation sets
// beta = alpha^H).  Grid (ceil(s*s/256), K).
template <typename T>
__global__ void k_circ_fwd(const cx<T>* h00, const cx<T>* v, int m, int ny, int nx, double gry, double grx,
                           cx<T>* hs, cx<T>* vs) {
  const int s = m / (ny * nx), na = m / ny;
  const int kb = blockIdx.y, i = kb / nx, j = kb % nx;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= s * s) return;
  const int r = e % s, c = e / s;
  double hr = 0.0, hi = 0.0, ar = 0.0, ai = 0.0;  // alpha_s(c, r) for vs(r, c) = conj(alpha_s(c, r))
  for (int l = 0; l < nx; ++l) {
    double h1r = 0.0, h1i = 0.0, a1r = 0.0, a1i = 0.0;
    for (int p = 0; p < ny; ++p) {
      double sn, cs;
      sincos(gry * (double)(i * p) / (double)ny, &sn, &cs);
      const size_t col_h = (size_t)p * na + (size_t)l * s + c;
      const cx<T> h = h00[r + col_h * m];
      h1r += pf::to_d(h.x) * cs - pf::to_d(h.y) * sn;
      h1i += pf::to_d(h.x) * sn + pf::to_d(h.y) * cs;
      // alpha(c, col) = conj(v(col, c)), col = p na + l s + r
      const size_t col_a = (size_t)p * na + (size_t)l * s + r;
      const cx<T> a = v[col_a + (size_t)c * m];
      const double xr = pf::to_d(a.x), xi = -pf::to_d(a.y);
      a1r += xr * cs - xi * sn;
      a1i += xr * sn + xi * cs;
    }
    double sn, cs;
    sincos(grx * (double)(j * l) / (double)nx, &sn, &cs);
    hr += h1r * cs - h1i * sn;
    hi += h1r * sn + h1i * cs;
    ar += a1r * cs - a1i * sn;
    ai += a1r * sn + a1i * cs;
  }
  hs[(size_t)kb * s * s + r + (size_t)c * s] = pf::mk<T>(T(hr), T(hi));
  vs[(size_t)kb * s * s + r + (size_t)c * s] = pf::mk<T>(T(ar), T(-ai));
}
// g_b = P1 diag_i(P2 diag_j(gs[b K + i nx + j]) P2^H) P1^H:
//   g((a nx + u) s + r, (a' nx + u') s + c)
//     = 1/K sum_i w_y^{i (a - a')} sum_j w_x^{j (u - u')} gs[b K + i nx + j](r, c)
// The phases w_y^{i d} (d = a - a' in (-ny, ny)) and w_x^{j d} are tabulated
// in shared memory first: ny (2 ny - 1) + nx (2 nx - 1) entries, at most
// kCircTab (the entry refuses larger cell counts).  Grid (ceil(m*m/256), batch).
constexpr int kCircTab = 2048;  // phase-table entries (complex double, 32 KB) of k_circ_back
template <typename T>
__global__ void k_circ_back(cx<T>* out, long long so, int ld, const cx<T>* gs, int m, int ny, int nx, double gry,
                            double grx) {
  __shared__ double2 tab[kCircTab];
  const int ty = ny * (2 * ny - 1), tx = nx * (2 * nx - 1);
  for (int t = threadIdx.x; t < ty + tx; t += blockDim.x) {
    double sn, cs;
    if (t < ty) {
      const int i = t / (2 * ny - 1), d = t % (2 * ny - 1) - (ny - 1);
      sincos(gry * (double)(i * d) / (double)ny, &sn, &cs);
    } else {
      const int u = t - ty, j = u / (2 * nx - 1), d = u % (2 * nx - 1) - (nx - 1);
      sincos(grx * (double)(j * d) / (double)nx, &sn, &cs);
    }
    tab[t] = make_double2(cs, sn);
  }
  __syncthreads();
  const int b = blockIdx.y;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * m) return;
  const int K = ny * nx, s = m / K;
  const int R = e % m, Cc = e / m;
  const int a = R / (nx * s), u = (R / s) % nx, r = R % s;
  const int a2 = Cc / (nx * s), u2 = (Cc / s) % nx, c = Cc % s;
  const cx<T>* g = gs + (size_t)b * K * s * s + r + (size_t)c * s;
  const double2* wy = tab + (a - a2 + ny - 1);
  const double2* wx = tab + ty + (u - u2 + nx - 1);
  double xr = 0.0, xi = 0.0;
  for (int i = 0; i < ny; ++i) {
    double yr = 0.0, yi = 0.0;
    for (int j = 0; j < nx; ++j) {
      const cx<T> v = g[(size_t)(i * nx + j) * s * s];
      const double2 w = wx[j * (2 * nx - 1)];
      yr += pf::to_d(v.x) * w.x - pf::to_d(v.y) * w.y;
      yi += pf::to_d(v.x) * w.y + pf::to_d(v.y) * w.x;
    }
    const double2 w = wy[i * (2 * ny - 1)];
    xr += yr * w.x - yi * w.y;
    xi += yr * w.y + yi * w.x;
  }
  out[(size_t)b * so + R + (size_t)Cc * ld] = pf::mk<T>(T(xr / K), T(xi / K));
}
// Small decimations of block-circulant leads with blocks of at most 48: the
// resident FP64 decimation of the n <= 48 kernels (transport.cuh), one CTA
// a small block with its matrices in shared memory, a persistent grid over
// the B K blocks; g = inv(z - es) of block i into gs + i s^2 (ld s).
constexpr int kCircThreads = 256;
constexpr int kCircGridCap = 1024;  // CTAs in flight: bounds the global scratch
struct CircLayout {
  int m, ld;
  size_t mat, smem;
};
inline CircLayout circ_layout(int s) {
  CircLayout l;
  l.m = s;
  l.ld = s | 1;
  l.mat = (size_t)l.ld * s;
  l.smem = pf::NSM * l.mat * 16 + 32 * sizeof(double) + 2 * (size_t)s * 16 + (size_t)s * sizeof(int) + 64 * sizeof(int);
  return l;
}
template <int S>
__global__ void __launch_bounds__(kCircThreads)
    k_circ_decimate(const cx<double>* hs, const cx<double>* vs, int K, int total, const cx<double>* z, double conv,
                    int max_iter, cx<double>* gs, int* it_s, int* st_s, char* gscr, CircLayout lay) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int s = lay.m;
  pf::Ctx<double> c;
  cx<double>* sm = reinterpret_cast<cx<double>*>(smem_raw);
  for (int i = 0; i < pf::NSM; ++i) c.sm[i] = sm + i * lay.mat;
  unsigned char* tail = reinterpret_cast<unsigned char*>(sm + pf::NSM * lay.mat);
  c.red = reinterpret_cast<double*>(tail);
  c.iw.rowk = reinterpret_cast<cx<double>*>(tail + 32 * sizeof(double));
  c.iw.colk = c.iw.rowk + s;
  int* ip = reinterpret_cast<int*>(c.iw.colk + s);
  c.iw.perm = ip;
  c.iw.flag = ip + s;
  cx<double>* g = reinterpret_cast<cx<double>*>(gscr) + (size_t)blockIdx.x * pf::NG * lay.mat;
  for (int i = 0; i < pf::NG; ++i) c.gs[i] = g + i * lay.mat;
  c.ld = lay.ld;
  for (int i = blockIdx.x; i < total; i += gridDim.x) {
    const size_t kb = (size_t)(i % K) * s * s;
    int it = 0;
    // alpha = vs^H, beta = vs (util.f90 decimation: beta = alpha^H)
    const int st = pf::decimate<double, S>(c, s, z[i / K], pf::opN<double>(hs + kb, s), pf::opC<double>(vs + kb, s),
                                           pf::opN<double>(vs + kb, s), conv, max_iter, &it);
    pf::copy_out(gs + (size_t)i * s * s, s, false, c.sm[2], c.ld, s, s);
    if (threadIdx.x == 0) {
      it_s[i] = it;
      st_s[i] = st;
    }
    __syncthreads();
  }
}
// zs[b K + k] = z[b]; st_s = 0
template <typename T>
__global__ void k_circ_points(const cx<T>* z, int B, int K, cx<T>* zs, int* st_s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * K) return;
  zs[i] = z[i / K];
  st_s[i] = 0;
}
// per point: iterations = the most of its K small decimations, status = their OR
__global__ void k_circ_fold(const int* it_s, const int* st_s, int B, int K, int* it, int* st) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  int mx = 0, f = 0;
  for (int k = 0; k < K; ++k) {
    mx = max(mx, it_s[b * K + k]);
    f |= st_s[b * K + k];
  }
  it[b] = mx;
  st[b] |= f;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// Block-circulant leads: ny x nx Bloch cells (n_bloch_y, n_bloch_x) and the
// G.R products of the y and x lattice vectors of each lead (forward
// transforms); the back transform uses the left lead's, as the reference
// builds P1, P2 once from the left lead (negf/phinfortran.f90:622-628).
struct Circ {
  int ny = 1, nx = 1;
  double gr_l[2] = {0.0, 0.0};
  double gr_r[2] = {0.0, 0.0};
  int K() const { return ny * nx; }
};

struct TLayout {
  int n, nl, nr, m, nb, batch;
  size_t mat;  // elements per working matrix (m * m, ld m)
};

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

TLayout tlayout(int n, int nl, int nr, int npts, size_t cxb, bool tc = false) {
  TLayout l;
  l.n = n;
  l.nl = nl;
  l.nr = nr;
  l.m = std::max(n, std::max(nl, nr));
  l.mat = (size_t)l.m * l.m;
  int nb = g_tune_panel > 0 ? g_tune_panel : 32;
  while (nb > 4 && ((size_t)l.m * nb + l.m) * cxb > kPanelBytes) nb >>= 1;
  l.nb = nb;
  size_t per_point = (kMats * l.mat + 2 * (size_t)l.m * nb + (size_t)nb * nb + 8) * cxb + (size_t)l.m * 4 + 64;
  if (tc) per_point += pf::tc::zgemm_workspace(l.m, l.m, l.m, 1, false, false);
  size_t b = kBatchBytes / per_point;
  if (b < 1) b = 1;
  if (b > (size_t)kMaxBatch) b = kMaxBatch;
  if (g_tune_batch > 0 && (size_t)g_tune_batch < b) b = g_tune_batch;
  if (npts > 0 && (size_t)npts < b) b = npts;
  l.batch = (int)b;
  return l;
}

// global scratch of the resident small decimations (0: blocks above 48,
// which go through the batched small-block engine)
size_t circ_scratch_bytes(int sb) {
  if (sb > PF_NMAX_RESIDENT) return 0;
  return round256((size_t)kCircGridCap * pf::NG * circ_layout(sb).mat * 16);
}

// tlayout with the batch bounded so that the small-block batch of
// block-circulant leads (batch K) stays within one grid dimension
TLayout tiled_layout(int n, int nl, int nr, int npts, size_t cxb, bool tc, int K) {
  TLayout l = tlayout(n, nl, nr, npts, cxb, tc);
  if (K > 1) l.batch = std::max(1, std::min(l.batch, 65535 / K));
  return l;
}
// layout of the small-block engine: blocks of nl / K, batch K times the main
TLayout small_layout(const TLayout& L, int K, size_t cxb) {
  const int sb = L.nl / K;
  TLayout S = tlayout(sb, sb, sb, 0, cxb, false);
  S.batch = L.batch * K;
  return S;
}

template <typename T>
struct Work {
  cx<T>* mats[kMats];  // each [batch] matrices of mat elements
  cx<T>* P;
  cx<T>* W;
  cx<T>* M11;
  cx<T>* zl;
  cx<T>* zr;
  cx<T>* zd;
  int* piv;
  int* idx;
  int* active;
  int* itl;
  int* itr;
  int* st;
  int* counter;
};

// Carves the workspace (base == nullptr: only counts the bytes).
template <typename T>
size_t carve(char* base, const TLayout& L, Work<T>* w) {
  const size_t cxb = sizeof(cx<T>);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* r = base ? base + off : nullptr;
    off += round256(bytes);
    return r;
  };
  const size_t B = (size_t)L.batch;
  w->counter = reinterpret_cast<int*>(take(256));
  w->idx = reinterpret_cast<int*>(take(B * 4));
  w->active = reinterpret_cast<int*>(take(B * 4));
  w->itl = reinterpret_cast<int*>(take(B * 4));
  w->itr = reinterpret_cast<int*>(take(B * 4));
  w->st = reinterpret_cast<int*>(take(B * 4));
  w->zl = reinterpret_cast<cx<T>*>(take(B * cxb));
  w->zr = reinterpret_cast<cx<T>*>(take(B * cxb));
  w->zd = reinterpret_cast<cx<T>*>(take(B * cxb));
  w->piv = reinterpret_cast<int*>(take(B * L.m * 4));
  for (int i = 0; i < kMats; ++i) w->mats[i] = reinterpret_cast<cx<T>*>(take(B * L.mat * cxb));
  w->P = reinterpret_cast<cx<T>*>(take(B * L.m * L.nb * cxb));
  w->W = reinterpret_cast<cx<T>*>(take(B * L.m * L.nb * cxb));
  w->M11 = reinterpret_cast<cx<T>*>(take(B * L.nb * L.nb * cxb));
  return off;
}

template <typename T>
struct Engine {
  cudaStream_t s;
  int B;  // points in flight
  TLayout L;
  Work<T> w;
  int* host_count;
  // tensor-core products (FP64 engine only): slice workspace and the
  // product kernel's error flag
  bool tc = false;
  void* tcw = nullptr;
  size_t tcw_bytes = 0;
  int* tcerr = nullptr;
  // block-circulant leads: the option and the engine of the small blocks
  // (batch B K, FP64 or double-float SIMT products)
  const Circ* circ = nullptr;
  Engine<T>* small = nullptr;
  char* circ_scr = nullptr;  // scratch of the resident small decimations (FP64, blocks <= 48)

  dim3 eg(int elems) const { return dim3((elems + 255) / 256, B); }

  cudaError_t gemm(int m, int n, int k, const cx<T>* A, int lda, long long sA, bool ca, const cx<T>* Bm, int ldb,
                   long long sB, bool cb, cx<T>* C, int ldc, long long sC, cx<T> alpha, cx<T> beta,
                   const int* active, const cx<T>* zdiag = nullptr, const cx<T>* H = nullptr, int ldh = 0,
                   long long sH = 0) {
    if (m <= 0 || n <= 0) return cudaSuccess;
    if constexpr (std::is_same<T, double>::value) {
      if (tc) {
        if (alpha.y != 0.0 || beta.y != 0.0) return cudaErrorInvalidValue;
        pf::tc::ZgemmArgs a{};
        a.m = m;
        a.n = n;
        a.k = k;
        a.A = A;
        a.lda = lda;
        a.sA = sA;
        a.ca = ca;
        a.B = Bm;
        a.ldb = ldb;
        a.sB = sB;
        a.cb = cb;
        a.C = C;
        a.ldc = ldc;
        a.sC = sC;
        a.alpha = alpha.x;
        a.beta = beta.x;
        a.batch = B;
        a.active = active;
        a.zdiag = zdiag;
        a.H = H;
        a.ldh = ldh;
        a.sH = sH;
        return pf::tc::zgemm(a, tcw, tcw_bytes, tcerr, s);
      }
    }
    GemmArgs<T> g;
    g.m = m;
    g.n = n;
    g.k = k;
    g.A = A;
    g.lda = lda;
    g.sA = sA;
    g.B = Bm;
    g.ldb = ldb;
    g.sB = sB;
    g.C = C;
    g.ldc = ldc;
    g.sC = sC;
    g.alpha = alpha;
    g.beta = beta;
    g.active = active;
    g.zdiag = zdiag;
    g.H = H;
    g.ldh = ldh;
    g.sH = sH;
    const dim3 grid((m + BM - 1) / BM, (n + BN - 1) / BN, B);
    if (!ca && !cb)
      bgemm<T, false, false><<<grid, GT, 0, s>>>(g);
    else if (ca && !cb)
      bgemm<T, true, false><<<grid, GT, 0, s>>>(g);
    else if (!ca && cb)
      bgemm<T, false, true><<<grid, GT, 0, s>>>(g);
    else
      bgemm<T, true, true><<<grid, GT, 0, s>>>(g);
    return cudaGetLastError();
  }

  // In-place inverse of the n x n leading block of every matrix of A.
  int inverse(cx<T>* A, int n, const int* active) {
    const int ld = L.m;
    const long long sA = (long long)L.mat;
    const size_t small = ((size_t)(n | 1) * n + 2 * (size_t)n) * sizeof(cx<T>) + ((size_t)n + 1) * 4;
    if (small <= kSmallInvBytes) {
      TL_CUDA(cudaFuncSetAttribute(inv_small<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)small));
      inv_small<T><<<B, 256, small, s>>>(A, ld, sA, n, active, w.st);
      TL_CUDA(cudaGetLastError());
      return PF_SUCCESS;
    }
    const int nb = L.nb;
    const size_t psm = ((size_t)n * nb + n) * sizeof(cx<T>);
    TL_CUDA(cudaFuncSetAttribute(gje_panel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm));
    const cx<T> one = hc<T>(1.0), zero = hc<T>(0.0);
    for (int k = 0; k < n; k += nb) {
      const int kb = std::min(nb, n - k);
      gje_panel<T><<<B, 256, psm, s>>>(A, ld, sA, n, k, kb, w.piv, w.P, w.M11, active, w.st);
      gje_swap<T><<<dim3((n + 255) / 256, B), 256, 0, s>>>(A, ld, sA, n, k, kb, w.piv, w.W, active);
      const long long sP = (long long)n * kb, sW = (long long)kb * n, sM = (long long)kb * kb;
      // rows above and below the pivot rows: += (factored panel rows) W
      TL_CUDA(gemm(k, n, kb, w.P, n, sP, false, w.W, kb, sW, false, A, ld, sA, one, one, active));
      TL_CUDA(gemm(n - k - kb, n, kb, w.P + (k + kb), n, sP, false, w.W, kb, sW, false, A + (k + kb), ld, sA, one,
                   one, active));
      // pivot rows: = M11 W
      TL_CUDA(gemm(kb, n, kb, w.M11, kb, sM, false, w.W, kb, sW, false, A + k, ld, sA, one, zero, active));
      gje_restore<T><<<dim3((n * kb + 255) / 256, B), 256, 0, s>>>(A, ld, sA, n, k, kb, w.P, active);
    }
    gje_unpermute<T><<<B, 256, 0, s>>>(A, ld, sA, n, w.piv, active);
    TL_CUDA(cudaGetLastError());
    return PF_SUCCESS;
  }

  // Lopez-Sancho decimation of one lead for the batch (surface.f90:479-497)
  // with alpha0 = v^H, beta0 = v; g = inv(z - es) into out.
  // h00 and v: one shared block (ss = 0) or per point b the block b mod
  // period at stride ss, leading dimension lds.
  int decimate(int m, const cx<T>* h00, const cx<T>* v, const cx<T>* z, double conv, int max_iter, int* it,
               cx<T>* out, long long ss = 0, int period = 1, int lds = 0) {
    if (lds <= 0) lds = m;
    const int ld = L.m;
    const long long sm = (long long)L.mat;
    cx<T>* al = w.mats[0];
    cx<T>* be = w.mats[1];
    cx<T>* e1 = w.mats[2];
    cx<T>* es = w.mats[3];
    cx<T>* W1 = w.mats[4];
    cx<T>* A2 = w.mats[5];
    cx<T>* B2 = w.mats[6];
    cx<T>* TT = w.mats[7];
    cx<T>* aln = w.mats[8];
    cx<T>* ben = w.mats[9];
    const cx<T> one = hc<T>(1.0), zero = hc<T>(0.0);
    k_copy_per<T><<<eg(m * m), 256, 0, s>>>(e1, sm, h00, ss, period, lds, m, m, ld, 0);
    k_copy_per<T><<<eg(m * m), 256, 0, s>>>(es, sm, h00, ss, period, lds, m, m, ld, 0);
    k_copy_per<T><<<eg(m * m), 256, 0, s>>>(al, sm, v, ss, period, lds, m, m, ld, 1);
    k_copy_per<T><<<eg(m * m), 256, 0, s>>>(be, sm, v, ss, period, lds, m, m, ld, 0);
    k_fill<<<(B + 255) / 256, 256, 0, s>>>(it, B, 0);
    k_fill<<<(B + 255) / 256, 256, 0, s>>>(w.active, B, 1);
    TL_CUDA(cudaGetLastError());
    int first = 1;
    for (;;) {
      k_fill<<<1, 32, 0, s>>>(w.counter, 1, 0);
      k_converge<T><<<B, 256, 0, s>>>(al, sm, m, ld, conv, max_iter, w.active, it, w.st, w.counter, first);
      first = 0;
      TL_CUDA(cudaGetLastError());
      TL_CUDA(cudaStreamSynchronize(s));
      TL_CUDA(cudaMemcpy(host_count, w.counter, sizeof(int), cudaMemcpyDeviceToHost));
      if (*host_count == 0) break;
      k_shift_neg<T><<<eg(m * m), 256, 0, s>>>(W1, e1, sm, m, ld, z, w.active);
      int rc = inverse(W1, m, w.active);
      if (rc) return rc;
      TL_CUDA(gemm(m, m, m, al, ld, sm, false, W1, ld, sm, false, A2, ld, sm, one, zero, w.active));
      TL_CUDA(gemm(m, m, m, be, ld, sm, false, W1, ld, sm, false, B2, ld, sm, one, zero, w.active));
      TL_CUDA(gemm(m, m, m, A2, ld, sm, false, be, ld, sm, false, TT, ld, sm, one, zero, w.active));
      k_add2<T><<<eg(m * m), 256, 0, s>>>(e1, es, TT, sm, m, ld, w.active);
      TL_CUDA(gemm(m, m, m, B2, ld, sm, false, al, ld, sm, false, e1, ld, sm, one, one, w.active));
      TL_CUDA(gemm(m, m, m, A2, ld, sm, false, al, ld, sm, false, aln, ld, sm, one, zero, w.active));
      TL_CUDA(gemm(m, m, m, B2, ld, sm, false, be, ld, sm, false, ben, ld, sm, one, zero, w.active));
      std::swap(al, aln);
      std::swap(be, ben);
    }
    k_shift_neg<T><<<eg(m * m), 256, 0, s>>>(out, es, sm, m, ld, z, nullptr);
    TL_CUDA(cudaGetLastError());
    return inverse(out, m, nullptr);
  }

  // Surface Green's function of one lead, g = inv(z - es) into out: the
  // decimation of the full matrices, or with block-circulant leads
  // circular_g (negf/circular.f90:42-105): transform, decimate the K small
  // blocks of every point as one batch of B K, transform back.
  int lead(int m, const cx<T>* h00, const cx<T>* v, const cx<T>* z, double conv, int max_iter, int* it, cx<T>* out,
           const double* gr_fwd) {
    if (!circ || circ->K() == 1) return decimate(m, h00, v, z, conv, max_iter, it, out);
    const int ny = circ->ny, nx = circ->nx, K = circ->K(), sb = m / K;
    Engine<T>& e = *small;
    e.B = B * K;
    const long long s2 = (long long)sb * sb;
    cx<T>* hs = e.w.mats[12];
    cx<T>* vs = e.w.mats[13];
    cx<T>* gs = e.w.mats[10];
    k_circ_fwd<T><<<dim3((unsigned)((s2 + 255) / 256), K), 256, 0, s>>>(h00, v, m, ny, nx, gr_fwd[0], gr_fwd[1], hs,
                                                                        vs);
    TL_CUDA(cudaGetLastError());
    bool resident = false;
    if constexpr (std::is_same<T, double>::value) resident = circ_scr != nullptr;
    if (resident) {
      if constexpr (std::is_same<T, double>::value) {
        const CircLayout cl = circ_layout(sb);
        const int Sx = (sb + 31) / 32;
        auto kfn = Sx == 1 ? k_circ_decimate<1> : k_circ_decimate<2>;
        TL_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cl.smem));
        int per_sm = 0, dev = 0, sms = 0;
        TL_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, kCircThreads, cl.smem));
        TL_CUDA(cudaGetDevice(&dev));
        TL_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if (per_sm < 1) return set_err(PF_ERR_SIZE, "pf_tiled_circ: small decimation does not fit on the device");
        const int grid = std::min(std::min(B * K, sms * per_sm), kCircGridCap);
        kfn<<<grid, kCircThreads, cl.smem, s>>>(hs, vs, K, B * K, z, conv, max_iter, gs, e.w.itl, e.w.st, circ_scr,
                                                cl);
        TL_CUDA(cudaGetLastError());
      }
    } else {
      k_circ_points<T><<<(B * K + 255) / 256, 256, 0, s>>>(z, B, K, e.w.zl, e.w.st);
      TL_CUDA(cudaGetLastError());
      int rc = e.decimate(sb, hs, vs, e.w.zl, conv, max_iter, e.w.itl, gs, s2, K, sb);
      if (rc) return rc;
    }
    k_circ_fold<<<(B + 255) / 256, 256, 0, s>>>(e.w.itl, e.w.st, B, K, it, w.st);
    k_circ_back<T><<<eg(m * m), 256, 0, s>>>(out, (long long)L.mat, L.m, gs, m, ny, nx, circ->gr_l[0],
                                             circ->gr_l[1]);
    TL_CUDA(cudaGetLastError());
    return PF_SUCCESS;
  }

  // One batch of points sharing block set q: leads, sweep, Caroli.
  int run(const pf::System<T>& sys, int q, const double* E, int cnt, double eta, double eta0, double devf,
          double conv, int max_iter, bool mirror, const int* zero_flag, double* transl, int* status, int* iters,
          double* transr = nullptr) {
    const int n = L.n, nl = L.nl, nr = L.nr, Ld = sys.L, ld = L.m;
    const long long sm = (long long)L.mat;
    const cx<T> one = hc<T>(1.0), zero = hc<T>(0.0), mone = hc<T>(-1.0);
    const cx<T>* HL = sys.HL + (size_t)q * nl * nl;
    const cx<T>* HLv = sys.HLv + (size_t)q * nl * nl;
    const cx<T>* HR = sys.HR + (size_t)q * nr * nr;
    const cx<T>* HRv = sys.HRv + (size_t)q * nr * nr;
    const cx<T>* Hd = sys.Hd + (size_t)q * Ld * n * n;
    const cx<T>* Hdv = sys.Hdv + (size_t)q * (Ld > 1 ? Ld - 1 : 0) * n * n;
    const cx<T>* Hld = sys.Hld + (size_t)q * nl * n;
    const cx<T>* Hrd = sys.Hrd + (size_t)q * nr * n;
    k_points<T><<<(cnt + 127) / 128, 128, 0, s>>>(E, w.idx, cnt, eta, eta0, devf, w.zl, w.zr, w.zd, w.st);
    TL_CUDA(cudaGetLastError());
    cx<T>* gl = w.mats[10];
    cx<T>* sl = w.mats[11];
    cx<T>* gml = w.mats[12];
    cx<T>* gr = w.mats[13];
    cx<T>* sr = w.mats[14];
    cx<T>* gmr = w.mats[15];
    cx<T>* t0 = w.mats[0];
    cx<T>* t1 = w.mats[1];
    cx<T>* t2 = w.mats[2];
    int rc;
    // ---- left lead, advanced: z = E - i eps, alpha0 = Hlv^H, beta0 = Hlv
    if ((rc = lead(nl, HL, HLv, w.zl, conv, max_iter, w.itl, t1, circ ? circ->gr_l : nullptr))) return rc;
    TL_CUDA(gemm(nl, nl, nl, t1, ld, sm, false, HLv, nl, 0, false, t0, ld, sm, one, zero, nullptr));  // g V
    TL_CUDA(gemm(nl, nl, nl, HLv, nl, 0, true, t0, ld, sm, false, t2, ld, sm, one, zero, nullptr));   // sl_adv
    // wrapper conversions (lesser.f90:141-144): gl = gl_adv^H, sl = sl_adv^H, gml = -gml_adv
    k_copy<T><<<eg(nl * nl), 256, 0, s>>>(gl, sm, t1, sm, ld, nl, nl, ld, 1);
    k_copy<T><<<eg(nl * nl), 256, 0, s>>>(sl, sm, t2, sm, ld, nl, nl, ld, 1);
    k_gamma<T><<<eg(nl * nl), 256, 0, s>>>(gml, t2, sm, nl, ld, -1);
    TL_CUDA(cudaGetLastError());
    // ---- right lead, retarded: z = E + i eps
    if (mirror) {
      // identical leads: gr_ret = gl_adv^H, sr_ret = sl_adv^H, gmr_ret = -gml_adv
      k_copy<T><<<eg(nr * nr), 256, 0, s>>>(gr, sm, gl, sm, ld, nr, nr, ld, 0);
      k_copy<T><<<eg(nr * nr), 256, 0, s>>>(sr, sm, sl, sm, ld, nr, nr, ld, 0);
      k_copy<T><<<eg(nr * nr), 256, 0, s>>>(gmr, sm, gml, sm, ld, nr, nr, ld, 0);
      TL_CUDA(cudaMemcpyAsync(w.itr, w.itl, sizeof(int) * B, cudaMemcpyDeviceToDevice, s));
    } else {
      if ((rc = lead(nr, HR, HRv, w.zr, conv, max_iter, w.itr, gr, circ ? circ->gr_r : nullptr))) return rc;
      TL_CUDA(gemm(nr, nr, nr, gr, ld, sm, false, HRv, nr, 0, false, t0, ld, sm, one, zero, nullptr));
      TL_CUDA(gemm(nr, nr, nr, HRv, nr, 0, true, t0, ld, sm, false, sr, ld, sm, one, zero, nullptr));
      k_gamma<T><<<eg(nr * nr), 256, 0, s>>>(gmr, sr, sm, nr, ld, 1);
    }
    TL_CUDA(cudaGetLastError());
    // ---- left-to-right sweep (lesser.f90:547-654)
    cx<T>* g = w.mats[0];
    cx<T>* A = w.mats[1];
    cx<T>* T1 = w.mats[2];
    cx<T>* G0N = w.mats[3];
    cx<T>* U = w.mats[4];
    // layer 1: T1 = gl Hld (nl x n); g = inv(zD - Hd_1 - Hld^H T1); G0N = T1 g
    TL_CUDA(gemm(nl, n, nl, gl, ld, sm, false, Hld, nl, 0, false, T1, ld, sm, one, zero, nullptr));
    TL_CUDA(gemm(n, n, nl, Hld, nl, 0, true, T1, ld, sm, false, g, ld, sm, mone, zero, nullptr, w.zd, Hd, n, 0));
    if ((rc = inverse(g, n, nullptr))) return rc;
    TL_CUDA(gemm(nl, n, n, T1, ld, sm, false, g, ld, sm, false, G0N, ld, sm, one, zero, nullptr));
    for (int i = 1; i < Ld; ++i) {
      const cx<T>* V = Hdv + (size_t)(i - 1) * n * n;
      TL_CUDA(gemm(n, n, n, g, ld, sm, false, V, n, 0, false, T1, ld, sm, one, zero, nullptr));
      TL_CUDA(gemm(n, n, n, V, n, 0, true, T1, ld, sm, false, A, ld, sm, mone, zero, nullptr, w.zd,
                   Hd + (size_t)i * n * n, n, 0));
      if ((rc = inverse(A, n, nullptr))) return rc;
      TL_CUDA(gemm(nl, n, n, G0N, ld, sm, false, V, n, 0, false, U, ld, sm, one, zero, nullptr));
      TL_CUDA(gemm(nl, n, n, U, ld, sm, false, A, ld, sm, false, G0N, ld, sm, one, zero, nullptr));
      std::swap(g, A);
    }
    // right closure: A = inv(zD - HR - sr - Hrd g Hrd^H); G_{0,N+1} = G0N Hrd^H A
    TL_CUDA(gemm(n, nr, n, g, ld, sm, false, Hrd, nr, 0, true, T1, ld, sm, one, zero, nullptr));
    TL_CUDA(gemm(nr, nr, n, Hrd, nr, 0, false, T1, ld, sm, false, A, ld, sm, mone, zero, nullptr, w.zd, HR, nr, 0));
    k_sub<T><<<eg(nr * nr), 256, 0, s>>>(A, sr, sm, nr, ld);
    if ((rc = inverse(A, nr, nullptr))) return rc;
    TL_CUDA(gemm(nl, nr, n, G0N, ld, sm, false, Hrd, nr, 0, true, U, ld, sm, one, zero, nullptr));
    TL_CUDA(gemm(nl, nr, nr, U, ld, sm, false, A, ld, sm, false, T1, ld, sm, one, zero, nullptr));  // G_D_LR
    // Caroli: Re Tr[(G gmr)(G^H gml)]
    TL_CUDA(gemm(nl, nr, nr, T1, ld, sm, false, gmr, ld, sm, false, U, ld, sm, one, zero, nullptr));
    TL_CUDA(gemm(nr, nl, nl, T1, ld, sm, true, gml, ld, sm, false, g, ld, sm, one, zero, nullptr));
    k_trace<T><<<cnt, 256, 0, s>>>(U, g, sm, nl, nr, ld, w.idx, zero_flag, w.st, w.itl, w.itr, transl, status,
                                   iters);
    TL_CUDA(cudaGetLastError());
    if (!transr) return PF_SUCCESS;
    // ---- right-to-left sweep (lesser.f90:694-784), T_R (:794-800)
    // layer N: T1 = gr Hrd (nr x n); g = inv(zD - Hd_N - Hrd^H T1); GNo = T1 g
    TL_CUDA(gemm(nr, n, nr, gr, ld, sm, false, Hrd, nr, 0, false, T1, ld, sm, one, zero, nullptr));
    TL_CUDA(gemm(n, n, nr, Hrd, nr, 0, true, T1, ld, sm, false, g, ld, sm, mone, zero, nullptr, w.zd,
                 Hd + (size_t)(Ld - 1) * n * n, n, 0));
    if ((rc = inverse(g, n, nullptr))) return rc;
    TL_CUDA(gemm(nr, n, n, T1, ld, sm, false, g, ld, sm, false, G0N, ld, sm, one, zero, nullptr));
    for (int i = Ld - 1; i >= 1; --i) {
      // V = Hdv_i^H couples layer i + 1 to layer i
      const cx<T>* V = Hdv + (size_t)(i - 1) * n * n;
      TL_CUDA(gemm(n, n, n, g, ld, sm, false, V, n, 0, true, T1, ld, sm, one, zero, nullptr));
      TL_CUDA(gemm(n, n, n, V, n, 0, false, T1, ld, sm, false, A, ld, sm, mone, zero, nullptr, w.zd,
                   Hd + (size_t)(i - 1) * n * n, n, 0));
      if ((rc = inverse(A, n, nullptr))) return rc;
      TL_CUDA(gemm(nr, n, n, G0N, ld, sm, false, V, n, 0, true, U, ld, sm, one, zero, nullptr));
      TL_CUDA(gemm(nr, n, n, U, ld, sm, false, A, ld, sm, false, G0N, ld, sm, one, zero, nullptr));
      std::swap(g, A);
    }
    // left closure: A = inv(zD - HL - sl - Hld g Hld^H); G_{N+1,0} = GNo Hld^H A
    TL_CUDA(gemm(n, nl, n, g, ld, sm, false, Hld, nl, 0, true, T1, ld, sm, one, zero, nullptr));
    TL_CUDA(gemm(nl, nl, n, Hld, nl, 0, false, T1, ld, sm, false, A, ld, sm, mone, zero, nullptr, w.zd, HL, nl, 0));
    k_sub<T><<<eg(nl * nl), 256, 0, s>>>(A, sl, sm, nl, ld);
    if ((rc = inverse(A, nl, nullptr))) return rc;
    TL_CUDA(gemm(nr, nl, n, G0N, ld, sm, false, Hld, nl, 0, true, U, ld, sm, one, zero, nullptr));
    TL_CUDA(gemm(nr, nl, nl, U, ld, sm, false, A, ld, sm, false, T1, ld, sm, one, zero, nullptr));  // G_D_RL
    // Caroli: Re Tr[(G_D_RL gml)(G_D_RL^H gmr)]
    TL_CUDA(gemm(nr, nl, nl, T1, ld, sm, false, gml, ld, sm, false, U, ld, sm, one, zero, nullptr));
    TL_CUDA(gemm(nl, nr, nr, T1, ld, sm, true, gmr, ld, sm, false, g, ld, sm, one, zero, nullptr));
    k_trace<T><<<cnt, 256, 0, s>>>(U, g, sm, nr, nl, ld, w.idx, zero_flag, w.st, w.itl, w.itr, transr, status,
                                   nullptr);
    TL_CUDA(cudaGetLastError());
    return PF_SUCCESS;
  }
};

// bytes of one q's blocks converted to double-float (0 for FP64)
size_t conv_bytes(int n, int nl, int nr, int L, int arith) {
  if (arith != PF_ARITH_DF64) return 0;
  const size_t c = 2 * (size_t)nl * nl + 2 * (size_t)nr * nr + (size_t)L * n * n + (size_t)(L > 1 ? L - 1 : 0) * n * n +
                   (size_t)nl * n + (size_t)nr * n;
  return round256(c * 16);
}

// Driver shared by both arithmetics: group by q, (convert,) run batches.
template <typename T>
int drive(int n, int nl, int nr, int L, int nq, const double* const blk[8], int npts, const double* E,
          const int* qidx, const int* zero_flag, double eta, double eta0, double dev_factor, double convergence,
          int max_iter, double* transl, int* status, int* iters, char* base, size_t work_bytes, cudaStream_t st,
          int arith, const Circ* circ, double* transr) {
  Engine<T> e;
  const bool tc = arith == PF_ARITH_TC;
  const int K = circ ? circ->K() : 1;
  e.L = tiled_layout(n, nl, nr, npts, sizeof(cx<T>), tc, K);
  const size_t cb = conv_bytes(n, nl, nr, L, arith);
  const size_t tcb = tc ? pf::tc::zgemm_workspace(e.L.m, e.L.m, e.L.m, e.L.batch, false, false) : 0;
  size_t need = 256 + cb + carve<T>(nullptr, e.L, &e.w) + tcb;
  Engine<T> se;  // small blocks of block-circulant leads
  size_t scr = 0;
  if (K > 1) {
    se.L = small_layout(e.L, K, sizeof(cx<T>));
    need += round256(tcb) - tcb + carve<T>(nullptr, se.L, &se.w);
    if (std::is_same<T, double>::value) scr = circ_scratch_bytes(nl / K);
    need += scr;
  }
  if (!base || work_bytes < need) return set_err(PF_ERR_ARG, "pf_tiled: workspace too small");
  if (tc && !pf::tc::tma_available())
    return set_err(PF_ERR_CUDA, "pf_tiled: the driver provides no cuTensorMapEncodeTiled");
  int* mirror_dev = reinterpret_cast<int*>(base);  // 256-byte header: mirror flag, tensor-core error flag
  pf::df64* conv = reinterpret_cast<pf::df64*>(base + 256);
  const size_t wb = carve<T>(base + 256 + cb, e.L, &e.w);
  if (tc) {
    e.tc = true;
    e.tcw = base + 256 + cb + wb;
    e.tcw_bytes = tcb;
    e.tcerr = mirror_dev + 1;
    TL_CUDA(cudaMemsetAsync(e.tcerr, 0, sizeof(int), st));
  }
  e.s = st;
  int host_count = 0;
  e.host_count = &host_count;
  if (K > 1) {
    const size_t sw = carve<T>(base + 256 + cb + wb + round256(tcb), se.L, &se.w);
    if (scr) e.circ_scr = base + 256 + cb + wb + round256(tcb) + sw;
    se.s = st;
    se.host_count = &host_count;
    e.circ = circ;
    e.small = &se;
  }
  std::vector<int> q(npts, 0);
  if (qidx) {
    TL_CUDA(cudaStreamSynchronize(st));
    TL_CUDA(cudaMemcpy(q.data(), qidx, sizeof(int) * npts, cudaMemcpyDeviceToHost));
  }
  for (int i = 0; i < npts; ++i)
    if (q[i] < 0 || q[i] >= nq) return set_err(PF_ERR_ARG, "pf_tiled: qidx out of range");
  std::vector<int> order(npts);
  for (int i = 0; i < npts; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return q[a] < q[b]; });
  // per-q element counts of the eight block arrays (complex entries)
  const size_t cnt_q[8] = {(size_t)nl * nl, (size_t)nl * nl, (size_t)nr * nr, (size_t)nr * nr, (size_t)L * n * n,
                           (size_t)(L > 1 ? L - 1 : 0) * n * n, (size_t)nl * n, (size_t)nr * n};
  size_t i0 = 0;
  while (i0 < (size_t)npts) {
    const int qq = q[order[i0]];
    size_t i1 = i0;
    while (i1 < (size_t)npts && q[order[i1]] == qq) ++i1;
    bool mirror = false;
    if (nl == nr) {
      k_fill<<<1, 32, 0, st>>>(mirror_dev, 1, 0);
      const size_t off = (size_t)qq * nl * nl * 2;
      k_mirror<<<64, 256, 0, st>>>(blk[0] + off, blk[1] + off, blk[2] + off, blk[3] + off, (size_t)nl * nl * 2,
                                   mirror_dev);
      TL_CUDA(cudaGetLastError());
      TL_CUDA(cudaStreamSynchronize(st));
      int diff = 1;
      TL_CUDA(cudaMemcpy(&diff, mirror_dev, sizeof(int), cudaMemcpyDeviceToHost));
      mirror = (diff == 0);
    }
    // the block set of this q, in the engine's arithmetic
    pf::System<T> sys;
    sys.n = n;
    sys.nl = nl;
    sys.nr = nr;
    sys.L = L;
    sys.nq = 1;
    const cx<T>** dst[8] = {&sys.HL, &sys.HLv, &sys.HR, &sys.HRv, &sys.Hd, &sys.Hdv, &sys.Hld, &sys.Hrd};
    pf::df64* c = conv;
    for (int k = 0; k < 8; ++k) {
      const double* src = blk[k] ? blk[k] + 2 * cnt_q[k] * (size_t)qq : nullptr;
      if (arith == PF_ARITH_DF64) {
        if (cnt_q[k]) {
          const size_t nd = 2 * cnt_q[k];
          const unsigned g = (unsigned)std::min<size_t>((nd + 255) / 256, 4096);
          k_to_df64<<<g, 256, 0, st>>>(src, c, nd);
          TL_CUDA(cudaGetLastError());
        }
        *dst[k] = reinterpret_cast<const cx<T>*>(c);
        c += 2 * cnt_q[k];
      } else {
        *dst[k] = reinterpret_cast<const cx<T>*>(src);
      }
    }
    for (size_t c0 = i0; c0 < i1; c0 += (size_t)e.L.batch) {
      const int cnt = (int)std::min((size_t)e.L.batch, i1 - c0);
      if (!qidx) {
        k_iota<<<(cnt + 255) / 256, 256, 0, st>>>(e.w.idx, cnt, (int)c0);
        TL_CUDA(cudaGetLastError());
      } else {
        TL_CUDA(cudaStreamSynchronize(st));
        TL_CUDA(cudaMemcpy(e.w.idx, order.data() + c0, sizeof(int) * cnt, cudaMemcpyHostToDevice));
      }
      e.B = cnt;
      const int rc = e.run(sys, 0, E, cnt, eta, eta0, dev_factor, convergence, max_iter, mirror, zero_flag, transl,
                           status, iters, transr);
      if (rc) return rc;
    }
    i0 = i1;
  }
  TL_CUDA(cudaStreamSynchronize(st));
  if (tc) {
    int herr = 0;
    TL_CUDA(cudaMemcpy(&herr, e.tcerr, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) return set_err(PF_ERR_CUDA, "pf_tiled: a pipeline wait of the tensor-core product kernel timed out");
  }
  return PF_SUCCESS;
}

size_t tiled_bytes(int n, int nl, int nr, int L, int nq, int npts, int arith, int K) {
  if (n <= 0 || nl <= 0 || nr <= 0 || L <= 0 || nq <= 0 || npts < 0) return 0;
  if (n > PF_NMAX_TILED || nl > PF_NMAX_TILED || nr > PF_NMAX_TILED) return 0;
  if (arith != PF_ARITH_FP64 && arith != PF_ARITH_DF64 && arith != PF_ARITH_TC) return 0;
  const TLayout L2 = tiled_layout(n, nl, nr, npts, 16, arith == PF_ARITH_TC, K);
  const size_t cb = conv_bytes(n, nl, nr, L, arith);
  const size_t tcb = arith == PF_ARITH_TC ? pf::tc::zgemm_workspace(L2.m, L2.m, L2.m, L2.batch, false, false) : 0;
  size_t b = 256 + cb + tcb;
  if (arith != PF_ARITH_DF64) {
    Work<double> w;
    b += carve<double>(nullptr, L2, &w);
  } else {
    Work<pf::df64> w;
    b += carve<pf::df64>(nullptr, L2, &w);
  }
  if (K > 1) {
    const TLayout S = small_layout(L2, K, 16);
    Work<double> w;  // complex double and complex double-float have the same size
    b += round256(tcb) - tcb + carve<double>(nullptr, S, &w);
    if (arith != PF_ARITH_DF64) b += circ_scratch_bytes(nl / K);
  }
  return b;
}

// nullptr when (nl, nr, ny, nx) describe block-circulant leads
const char* circ_dims_error(int nl, int nr, int ny, int nx) {
  if (ny < 1 || nx < 1) return "pf_tiled_circ: n_bloch_y and n_bloch_x must be positive";
  if ((long long)ny * nx > 256) return "pf_tiled_circ: at most 256 Bloch cells";
  if ((long long)ny * (2 * ny - 1) + (long long)nx * (2 * nx - 1) > kCircTab)
    return "pf_tiled_circ: n_bloch_y, n_bloch_x too large for the phase table";
  if (nl != nr) return "pf_tiled_circ: block-circulant leads need nl == nr";
  if (nl <= 0 || nl % (ny * nx)) return "pf_tiled_circ: nl must be a multiple of n_bloch_y * n_bloch_x";
  return nullptr;
}

int tiled_entry(int n, int nl, int nr, int L, int nq, const double* const blk[8], int npts, const double* E,
                const int* qidx, const int* zero_flag, double eta, double eta0, double dev_factor, double convergence,
                int max_iter, int arith, const Circ* circ, double* transl, double* transr, int* status, int* iters,
                void* work, size_t work_bytes, void* stream) {
  if (n <= 0 || nl <= 0 || nr <= 0 || L <= 0 || nq <= 0 || npts < 0)
    return set_err(PF_ERR_ARG, "pf_tiled: dimensions must be positive");
  if (n > PF_NMAX_TILED || nl > PF_NMAX_TILED || nr > PF_NMAX_TILED)
    return set_err(PF_ERR_SIZE, "pf_tiled: block size exceeds PF_NMAX_TILED");
  for (int k = 0; k < 8; ++k)
    if (!blk[k] && !(k == 5 && L == 1)) return set_err(PF_ERR_ARG, "pf_tiled: null block pointer");
  if (!E || !transl || !status) return set_err(PF_ERR_ARG, "pf_tiled: null pointer");
  if (max_iter <= 0) return set_err(PF_ERR_ARG, "pf_tiled: max_iter must be positive");
  if (arith != PF_ARITH_FP64 && arith != PF_ARITH_DF64 && arith != PF_ARITH_TC)
    return set_err(PF_ERR_ARG, "pf_tiled: unknown arithmetic");
  if (npts == 0) return PF_SUCCESS;
  cudaStream_t st = (cudaStream_t)stream;
  char* base = reinterpret_cast<char*>(work);
  if (arith != PF_ARITH_DF64)
    return drive<double>(n, nl, nr, L, nq, blk, npts, E, qidx, zero_flag, eta, eta0, dev_factor, convergence,
                         max_iter, transl, status, iters, base, work_bytes, st, arith, circ, transr);
  return drive<pf::df64>(n, nl, nr, L, nq, blk, npts, E, qidx, zero_flag, eta, eta0, dev_factor, convergence,
                         max_iter, transl, status, iters, base, work_bytes, st, arith, circ, transr);
}

}  // namespace

extern "C" {

const char* pf_tiled_last_error(void) { return g_err; }

int pf_tiled_set_tuning(int panel, int batch) {
  if (panel != 0 && panel != 4 && panel != 8 && panel != 16 && panel != 32)
    return set_err(PF_ERR_ARG, "pf_tiled_set_tuning: panel must be 0, 4, 8, 16 or 32");
  if (batch < 0 || batch > kMaxBatch) return set_err(PF_ERR_ARG, "pf_tiled_set_tuning: batch must be in [0, 256]");
  g_tune_panel = panel;
  g_tune_batch = batch;
  return PF_SUCCESS;
}

int pf_tiled_layout(int n, int nl, int nr, int npts, int arith, int* panel, int* batch) {
  if (n <= 0 || nl <= 0 || nr <= 0 || npts < 0 || !panel || !batch)
    return set_err(PF_ERR_ARG, "pf_tiled_layout: bad arguments");
  if (arith != PF_ARITH_FP64 && arith != PF_ARITH_DF64 && arith != PF_ARITH_TC)
    return set_err(PF_ERR_ARG, "pf_tiled_layout: unknown arithmetic");
  const TLayout L2 = tlayout(n, nl, nr, npts, 16, arith == PF_ARITH_TC);
  *panel = L2.nb;
  *batch = L2.batch;
  return PF_SUCCESS;
}

size_t pf_transport_tdb_tiled_workspace_size(int n, int nl, int nr, int L, int nq, int npts, int arith) {
  return tiled_bytes(n, nl, nr, L, nq, npts, arith, 1);
}

int pf_transport_tdb_tiled_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                               const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                               const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                               const int* zero_flag, double eta, double eta0, double dev_factor, double convergence,
                               int max_iter, int arith, double* transl, int* status, int* iters, void* work,
                               size_t work_bytes, void* stream) {
  const double* blk[8] = {HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd};
  return tiled_entry(n, nl, nr, L, nq, blk, npts, E, qidx, zero_flag, eta, eta0, dev_factor, convergence, max_iter,
                     arith, nullptr, transl, nullptr, status, iters, work, work_bytes, stream);
}

size_t pf_transport_tdb_tiled_circ_workspace_size(int n, int nl, int nr, int L, int nq, int npts, int arith,
                                                  int n_bloch_y, int n_bloch_x) {
  if (circ_dims_error(nl, nr, n_bloch_y, n_bloch_x)) return 0;
  return tiled_bytes(n, nl, nr, L, nq, npts, arith, n_bloch_y * n_bloch_x);
}

int pf_transport_tdb_tiled_circ_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                                    const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                                    const double* Hld, const double* Hrd, int npts, const double* E,
                                    const int* qidx, const int* zero_flag, double eta, double eta0,
                                    double dev_factor, double convergence, int max_iter, int arith, int n_bloch_y,
                                    int n_bloch_x, const double* gr, double* transl, int* status, int* iters,
                                    void* work, size_t work_bytes, void* stream) {
  if (const char* why = circ_dims_error(nl, nr, n_bloch_y, n_bloch_x)) return set_err(PF_ERR_ARG, why);
  if (!gr) return set_err(PF_ERR_ARG, "pf_tiled_circ: null gr");
  return pf_transport_tdb_tiled_ex_dev(n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd, npts, E, qidx,
                                       zero_flag, eta, eta0, dev_factor, convergence, max_iter, arith, n_bloch_y,
                                       n_bloch_x, gr, transl, nullptr, status, iters, work, work_bytes, stream);
}

size_t pf_transport_tdb_tiled_ex_workspace_size(int n, int nl, int nr, int L, int nq, int npts, int arith,
                                                int n_bloch_y, int n_bloch_x) {
  if (n_bloch_y == 1 && n_bloch_x == 1) return tiled_bytes(n, nl, nr, L, nq, npts, arith, 1);
  return pf_transport_tdb_tiled_circ_workspace_size(n, nl, nr, L, nq, npts, arith, n_bloch_y, n_bloch_x);
}

int pf_transport_tdb_tiled_ex_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                                  const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                                  const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                                  const int* zero_flag, double eta, double eta0, double dev_factor,
                                  double convergence, int max_iter, int arith, int n_bloch_y, int n_bloch_x,
                                  const double* gr, double* transl, double* transr, int* status, int* iters,
                                  void* work, size_t work_bytes, void* stream) {
  if (const char* why = circ_dims_error(nl, nr, n_bloch_y, n_bloch_x)) {
    // one Bloch cell: no block-circulant option, any nl, nr
    if (!(n_bloch_y == 1 && n_bloch_x == 1)) return set_err(PF_ERR_ARG, why);
  }
  const bool circ_on = n_bloch_y * n_bloch_x > 1;
  if (circ_on && !gr) return set_err(PF_ERR_ARG, "pf_tiled_circ: null gr");
  Circ c;
  if (circ_on) {
    c.ny = n_bloch_y;
    c.nx = n_bloch_x;
    c.gr_l[0] = gr[0];
    c.gr_l[1] = gr[1];
    c.gr_r[0] = gr[2];
    c.gr_r[1] = gr[3];
    for (int i = 0; i < 4; ++i)
      if (!std::isfinite(gr[i])) return set_err(PF_ERR_ARG, "pf_tiled_circ: gr must be finite");
  }
  const double* blk[8] = {HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd};
  return tiled_entry(n, nl, nr, L, nq, blk, npts, E, qidx, zero_flag, eta, eta0, dev_factor, convergence, max_iter,
                     arith, circ_on ? &c : nullptr, transl, transr, status, iters, work, work_bytes, stream);
}

}  // extern "C"
