// extern "C" boundary of the GB300 NEGF transport engine.
//
// The entry points replace the per-(ie,ik) Fortran calls of the tdb
// transport loop (negf/phinfortran.f90:1196-1213):
//   surface_green_tdb_mpi  (negf/surface.f90:344-383)
//   get_G_full_tdb_mpi     (negf/lesser.f90:100-157)
// batched over every (omega, q) point of a shard.  Matrices are the
// reference's complex(kind=8) column-major blocks; all pointers are plain
// double* to interleaved (re, im) pairs.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "../../include/phinfortran_gb300.h"
#include "mixed.cuh"

using pf::cx;

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

#define PF_CUDA(call)                               \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return cuda_err(e_, #call); \
  } while (0)

constexpr int kThreads = 256;

// Layout of the per-CTA scratch: NG matrices of ld*m elements.
struct Layout {
  int m;         // max(n, nl, nr)
  int ld;        // odd leading dimension >= m
  size_t mat;    // elements per matrix
  size_t smem;   // dynamic shared memory bytes
  size_t per_cta_bytes;
};

template <typename R>
Layout make_layout(int n, int nl, int nr) {
  Layout l;
  l.m = n > nl ? n : nl;
  l.m = l.m > nr ? l.m : nr;
  l.ld = l.m | 1;
  l.mat = (size_t)l.ld * l.m;
  const size_t cxb = sizeof(cx<R>);
  l.smem = pf::NSM * l.mat * cxb + 32 * sizeof(double) + 2 * (size_t)l.m * cxb + (size_t)l.m * sizeof(int) +
           64 * sizeof(int);
  l.per_cta_bytes = (size_t)pf::NG * l.mat * cxb;
  return l;
}

template <typename R>
__device__ pf::Ctx<R> make_ctx(const Layout& lay, char* gscr_base) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pf::Ctx<R> c;
  cx<R>* s = reinterpret_cast<cx<R>*>(smem_raw);
  for (int i = 0; i < pf::NSM; ++i) c.sm[i] = s + i * lay.mat;
  // tail: 32 reduction words, then the pivot row/column vectors, then ints
  unsigned char* tail = reinterpret_cast<unsigned char*>(s + pf::NSM * lay.mat);
  c.red = reinterpret_cast<double*>(tail);
  c.iw.rowk = reinterpret_cast<cx<R>*>(tail + 32 * sizeof(double));
  c.iw.colk = c.iw.rowk + lay.m;
  int* ip = reinterpret_cast<int*>(c.iw.colk + lay.m);
  c.iw.perm = ip;
  c.iw.flag = ip + lay.m;
  cx<R>* g = reinterpret_cast<cx<R>*>(gscr_base) + (size_t)blockIdx.x * pf::NG * lay.mat;
  for (int i = 0; i < pf::NG; ++i) c.gs[i] = g + i * lay.mat;
  c.ld = lay.ld;
  return c;
}

// Fused persistent kernel: each CTA pulls points from a device work queue,
// runs both lead decimations, the left-to-right sweep (and optionally the
// right-to-left one) and the Caroli traces, and retires the point.
template <typename R, int S>
__global__ void __launch_bounds__(kThreads) transport_kernel(pf::System<R> sys, pf::Points pts,
                                                             pf::Params P, pf::Outputs out, Layout lay,
                                                             char* gscr, int* queue) {
  pf::Ctx<R> c = make_ctx<R>(lay, gscr);
  __shared__ int s_p;
  for (;;) {
    if (threadIdx.x == 0) s_p = atomicAdd(queue, 1);
    __syncthreads();
    const int p = s_p;
    __syncthreads();
    if (p >= pts.npts) break;
    const int q = pts.qidx ? pts.qidx[p] : 0;
    const double E = pts.E[p];
    int itl = 0, itr = 0;
    int st = pf::lead_pair<R, S>(c, sys, q, E, P, &itl, &itr);
    const double eps = E * P.eta + P.eta0;
    const cx<R> zD = pf::mk<R>(R(E), R(P.dev_factor * eps));
    double tl = 0, tr = 0;
    st |= pf::sweep_lr<R, S>(c, sys, q, zD, &tl);
    if (P.want_transr) st |= pf::sweep_rl<R, S>(c, sys, q, zD, &tr);
    if (threadIdx.x == 0) {
      const bool zero = pts.zero_flag && pts.zero_flag[p];
      double a = (double)tl, b = (double)tr;
      // lesser.f90:795-807: values below 1e-60 (a NaN is not) become 0; ie==1 -> 0
      if (zero || a < 1.0e-60) a = 0.0;
      if (zero || b < 1.0e-60) b = 0.0;
      out.transl[p] = a;
      if (out.transr) out.transr[p] = P.want_transr ? b : 0.0;
      out.status[p] = st;
      if (out.iters) {
        out.iters[2 * p] = itl;
        out.iters[2 * p + 1] = itr;
      }
    }
    __syncthreads();
  }
}

struct DevInfo {
  int sms = 0;
  size_t smem_optin = 0;
};

DevInfo device_info() {
  DevInfo d;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return d;
  cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
  int v = 0;
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  d.smem_optin = (size_t)v;
  return d;
}

template <typename R, int S>
int grid_for(const Layout& lay, int npts) {
  auto k = transport_kernel<R, S>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.smem) != cudaSuccess)
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, lay.smem) != cudaSuccess) return -1;
  if (per_sm < 1) return -1;
  DevInfo d = device_info();
  int g = d.sms * per_sm;
  return g < npts ? g : npts;
}

int check_dims(int n, int nl, int nr, int L, int nq, int npts) {
  if (n <= 0 || nl <= 0 || nr <= 0 || L <= 0 || nq <= 0 || npts < 0)
    return set_err(PF_ERR_ARG, "pf: dimensions must be positive");
  if (n > PF_NMAX_RESIDENT || nl > PF_NMAX_RESIDENT || nr > PF_NMAX_RESIDENT)
    return set_err(PF_ERR_SIZE, "pf: block size exceeds the shared-memory resident kernel limit");
  return PF_SUCCESS;
}

template <typename R>
int launch_transport(const pf::System<R>& sys, const pf::Points& pts, const pf::Params& P,
                     const pf::Outputs& out, void* work, size_t work_bytes, cudaStream_t stream) {
  const Layout lay = make_layout<R>(sys.n, sys.nl, sys.nr);
  DevInfo d = device_info();
  if (lay.smem > d.smem_optin) return set_err(PF_ERR_SIZE, "pf: working set exceeds shared memory");
  if (pts.npts == 0) return PF_SUCCESS;
  const int S = (lay.m + 31) / 32;
  int grid = (S == 1) ? grid_for<R, 1>(lay, pts.npts) : grid_for<R, 2>(lay, pts.npts);
  if (grid <= 0) return set_err(PF_ERR_SIZE, "pf: kernel does not fit on the device");
  const size_t need = 256 + (size_t)grid * lay.per_cta_bytes;
  if (!work || work_bytes < need) return set_err(PF_ERR_ARG, "pf: workspace too small");
  int* queue = reinterpret_cast<int*>(work);
  char* gscr = reinterpret_cast<char*>(work) + 256;
  PF_CUDA(cudaMemsetAsync(queue, 0, sizeof(int), stream));
  if (S == 1)
    transport_kernel<R, 1><<<grid, kThreads, lay.smem, stream>>>(sys, pts, P, out, lay, gscr, queue);
  else
    transport_kernel<R, 2><<<grid, kThreads, lay.smem, stream>>>(sys, pts, P, out, lay, gscr, queue);
  PF_CUDA(cudaGetLastError());
  return PF_SUCCESS;
}

template <typename R>
size_t workspace_bytes(int n, int nl, int nr, int npts) {
  const Layout lay = make_layout<R>(n, nl, nr);
  const int S = (lay.m + 31) / 32;
  int grid = (S == 1) ? grid_for<R, 1>(lay, npts > 0 ? npts : 1) : grid_for<R, 2>(lay, npts > 0 ? npts : 1);
  if (grid <= 0) return 0;
  return 256 + (size_t)grid * lay.per_cta_bytes;
}

pf::System<double> make_sys(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                            const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                            const double* Hld, const double* Hrd) {
  pf::System<double> s;
  s.n = n;
  s.nl = nl;
  s.nr = nr;
  s.L = L;
  s.nq = nq;
  s.HL = reinterpret_cast<const cx<double>*>(HL);
  s.HLv = reinterpret_cast<const cx<double>*>(HLv);
  s.HR = reinterpret_cast<const cx<double>*>(HR);
  s.HRv = reinterpret_cast<const cx<double>*>(HRv);
  s.Hd = reinterpret_cast<const cx<double>*>(Hd);
  s.Hdv = reinterpret_cast<const cx<double>*>(Hdv);
  s.Hld = reinterpret_cast<const cx<double>*>(Hld);
  s.Hrd = reinterpret_cast<const cx<double>*>(Hrd);
  return s;
}

// Grow-only device buffers used by the host-pointer entry point.
struct HostStage {
  std::mutex mu;
  void* buf = nullptr;
  size_t cap = 0;
  int dev = -1;
};
HostStage g_stage;


// ===========================================================================
// Mixed-precision path
// ===========================================================================
using pf::dcx;
using pf::fcx;

// FP64 -> df64 and FP32 copies of a block array (grid-stride)
__global__ void convert_blocks_kernel(const cx<double>* src, dcx* d, fcx* f, size_t count) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
    const cx<double> v = src[i];
    dcx a;
    a.x = pf::df64(v.x);
    a.y = pf::df64(v.y);
    d[i] = a;
    if (f) f[i] = pf::mk<float>(a.x.hi, a.y.hi);
  }
}

struct MixedLayout {
  Layout base;     // smem slots are df64-sized (16 B per complex)
  size_t smem;
  size_t per_cta;  // bytes of per-CTA scratch
  size_t blocks_d, blocks_f;  // bytes of converted block copies (per call)
  size_t cnt[8];   // complex elements per block family (all q)
};

MixedLayout make_mixed_layout(int n, int nl, int nr, int L, int nq) {
  MixedLayout m;
  m.base = make_layout<double>(n, nl, nr);
  const size_t mat = m.base.mat;
  m.smem = pf::NSM_M * mat * 16 + 32 * sizeof(double) + 2 * (size_t)m.base.m * 16 + (size_t)m.base.m * sizeof(int) +
           64 * sizeof(int);
  const size_t nslab = (size_t)(L + 2);
  m.per_cta = ((size_t)pf::NGM * mat * 16 + nslab * mat * (8 + 8 + 16) + mat * 8 + 255) & ~(size_t)255;
  const size_t c[8] = {(size_t)nq * nl * nl, (size_t)nq * nl * nl, (size_t)nq * nr * nr, (size_t)nq * nr * nr,
                       (size_t)nq * L * n * n, (size_t)nq * (L > 1 ? L - 1 : 0) * n * n, (size_t)nq * nl * n,
                       (size_t)nq * nr * n};
  size_t tot = 0;
  for (int i = 0; i < 8; ++i) {
    m.cnt[i] = c[i];
    tot += (c[i] * 16 + 255) & ~(size_t)255;
  }
  m.blocks_d = tot;
  size_t totf = 0;
  for (int i = 2; i < 8; ++i) totf += (c[i] * 8 + 255) & ~(size_t)255;  // HR, HRv(unused), Hd, Hdv, Hld, Hrd
  m.blocks_f = totf;
  return m;
}

template <int S>
__global__ void __launch_bounds__(kThreads) mixed_kernel(pf::MSys sys, pf::Points pts, pf::Params P, int nref,
                                                         pf::Outputs out, MixedLayout lay, char* scratch,
                                                         int* queue) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pf::MCtx c;
  const size_t mat = lay.base.mat;
  dcx* s = reinterpret_cast<dcx*>(smem_raw);
  for (int i = 0; i < pf::NSM_M; ++i) c.sm[i] = s + i * mat;
  unsigned char* tail = reinterpret_cast<unsigned char*>(s + pf::NSM_M * mat);
  c.red = reinterpret_cast<double*>(tail);
  c.iwd.rowk = reinterpret_cast<dcx*>(tail + 32 * sizeof(double));
  c.iwd.colk = c.iwd.rowk + lay.base.m;
  int* ip = reinterpret_cast<int*>(c.iwd.colk + lay.base.m);
  c.iwd.perm = ip;
  c.iwd.flag = ip + lay.base.m;
  c.iwf.rowk = reinterpret_cast<fcx*>(c.iwd.rowk);
  c.iwf.colk = reinterpret_cast<fcx*>(c.iwd.colk);
  c.iwf.perm = c.iwd.perm;
  c.iwf.flag = c.iwd.flag;
  char* base = scratch + (size_t)blockIdx.x * lay.per_cta;
  dcx* g = reinterpret_cast<dcx*>(base);
  for (int i = 0; i < pf::NGM; ++i) c.gs[i] = g + i * mat;
  const size_t nslab = (size_t)(sys.L + 2);
  c.xv = g + pf::NGM * mat;
  c.lu = reinterpret_cast<fcx*>(c.xv + nslab * mat);
  c.yv = c.lu + nslab * mat;
  c.fsr = c.yv + nslab * mat;
  c.ld = lay.base.ld;
  c.mat = mat;
  __shared__ int s_p;
  for (;;) {
    if (threadIdx.x == 0) s_p = atomicAdd(queue, 1);
    __syncthreads();
    const int p = s_p;
    __syncthreads();
    if (p >= pts.npts) break;
    const int q = pts.qidx ? pts.qidx[p] : 0;
    const double E = pts.E[p];
    int itl = 0, itr = 0;
    int st = pf::mixed_leads<S>(c, sys, q, E, P, &itl, &itr);
    const double eps = E * P.eta + P.eta0;
    const fcx zf = pf::mk<float>((float)E, (float)(P.dev_factor * eps));
    st |= pf::mixed_factor_solve<S>(c, sys, q, zf);
    const dcx zL = pf::mk<pf::df64>(pf::df64(E), pf::df64(eps));
    const dcx zD = pf::mk<pf::df64>(pf::df64(E), pf::df64(P.dev_factor * eps));
    for (int k = 0; k < nref; ++k) pf::mixed_refine<S>(c, sys, q, zL, zD);
    const double tl = pf::mixed_caroli<S>(c, sys);
    if (threadIdx.x == 0) {
      const bool zero = pts.zero_flag && pts.zero_flag[p];
      double a = tl;
      if (zero || a < 1.0e-60) a = 0.0;
      if (!(a == a)) st |= pf::PF_NAN;
      out.transl[p] = a;
      out.status[p] = st;
      if (out.iters) {
        out.iters[2 * p] = itl;
        out.iters[2 * p + 1] = itr;
      }
    }
    __syncthreads();
  }
}

template <int S>
int mixed_grid(const MixedLayout& lay, int npts) {
  auto k = mixed_kernel<S>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.smem) != cudaSuccess) return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, lay.smem) != cudaSuccess) return -1;
  if (per_sm < 1) return -1;
  DevInfo d = device_info();
  int g = d.sms * per_sm;
  return g < npts ? g : npts;
}

size_t mixed_workspace_bytes(int n, int nl, int nr, int L, int nq, int npts) {
  MixedLayout lay = make_mixed_layout(n, nl, nr, L, nq);
  const int S = (lay.base.m + 31) / 32;
  const int g = (S == 1) ? mixed_grid<1>(lay, npts > 0 ? npts : 1) : mixed_grid<2>(lay, npts > 0 ? npts : 1);
  if (g <= 0) return 0;
  return 256 + lay.blocks_d + lay.blocks_f + (size_t)g * lay.per_cta;
}
}  // namespace

extern "C" int pf_transport_tdb_dev(int, int, int, int, int, const double*, const double*, const double*,
                                    const double*, const double*, const double*, const double*, const double*, int,
                                    const double*, const int*, const int*, double, double, double, double, int, int,
                                    double*, double*, int*, int*, void*, size_t, void*);
extern "C" int pf_transport_tdb_mixed_dev(int, int, int, int, int, const double*, const double*, const double*,
                                          const double*, const double*, const double*, const double*,
                                          const double*, int, const double*, const int*, const int*, double,
                                          double, double, double, int, int, double*, int*, int*, void*, size_t,
                                          void*);
namespace {
int host_run(bool mixed, int refine_iters, int n, int nl, int nr, int L, int nq, const double* HL,
             const double* HLv, const double* HR, const double* HRv, const double* Hd, const double* Hdv,
             const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
             const int* zero_flag, double eta, double eta0, double dev_factor, double convergence, int max_iter,
             int want_transr, double* transl, double* transr, int* status, int* iters) {
  int rc = check_dims(n, nl, nr, L, nq, npts);
  if (rc != PF_SUCCESS) return rc;
  if (!E || !transl || !status || (want_transr && !transr))
    return set_err(PF_ERR_ARG, "pf: null energy/output pointer");
  if (npts == 0) return PF_SUCCESS;
  std::lock_guard<std::mutex> lock(g_stage.mu);
  const size_t c16 = 16;
  const size_t b_HL = (size_t)nq * nl * nl * c16, b_HR = (size_t)nq * nr * nr * c16;
  const size_t b_Hd = (size_t)nq * L * n * n * c16, b_Hdv = (size_t)nq * (L - 1) * n * n * c16;
  const size_t b_Hld = (size_t)nq * nl * n * c16, b_Hrd = (size_t)nq * nr * n * c16;
  const size_t b_E = (size_t)npts * 8, b_i = (size_t)npts * 4;
  const size_t ws = mixed ? mixed_workspace_bytes(n, nl, nr, L, nq, npts)
                          : workspace_bytes<double>(n, nl, nr, npts);
  if (ws == 0) return set_err(PF_ERR_SIZE, "pf: kernel does not fit on the device");
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t total = al(b_HL) * 2 + al(b_HR) * 2 + al(b_Hd) + al(b_Hdv) + al(b_Hld) + al(b_Hrd) + al(b_E) +
                       al(b_i) * 2 + al(b_E) * 2 + al(b_i) + al(2 * b_i) + al(ws);
  int dev = 0;
  PF_CUDA(cudaGetDevice(&dev));
  if (g_stage.cap < total || g_stage.dev != dev) {
    if (g_stage.buf) cudaFree(g_stage.buf);
    g_stage.buf = nullptr;
    g_stage.cap = 0;
    PF_CUDA(cudaMalloc(&g_stage.buf, total));
    g_stage.cap = total;
    g_stage.dev = dev;
  }
  char* p = reinterpret_cast<char*>(g_stage.buf);
  auto take = [&](size_t b) {
    char* r = p;
    p += al(b);
    return r;
  };
  double* dHL = (double*)take(b_HL);
  double* dHLv = (double*)take(b_HL);
  double* dHR = (double*)take(b_HR);
  double* dHRv = (double*)take(b_HR);
  double* dHd = (double*)take(b_Hd);
  double* dHdv = (double*)take(b_Hdv);
  double* dHld = (double*)take(b_Hld);
  double* dHrd = (double*)take(b_Hrd);
  double* dE = (double*)take(b_E);
  int* dq = (int*)take(b_i);
  int* dz = (int*)take(b_i);
  double* dTL = (double*)take(b_E);
  double* dTR = (double*)take(b_E);
  int* dst = (int*)take(b_i);
  int* dit = (int*)take(2 * b_i);
  void* dws = take(ws);
  cudaStream_t s = 0;
  PF_CUDA(cudaMemcpyAsync(dHL, HL, b_HL, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dHLv, HLv, b_HL, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dHR, HR, b_HR, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dHRv, HRv, b_HR, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dHd, Hd, b_Hd, cudaMemcpyHostToDevice, s));
  if (L > 1) PF_CUDA(cudaMemcpyAsync(dHdv, Hdv, b_Hdv, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dHld, Hld, b_Hld, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dHrd, Hrd, b_Hrd, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dE, E, b_E, cudaMemcpyHostToDevice, s));
  if (qidx) PF_CUDA(cudaMemcpyAsync(dq, qidx, b_i, cudaMemcpyHostToDevice, s));
  if (zero_flag) PF_CUDA(cudaMemcpyAsync(dz, zero_flag, b_i, cudaMemcpyHostToDevice, s));
  if (mixed)
    rc = pf_transport_tdb_mixed_dev(n, nl, nr, L, nq, dHL, dHLv, dHR, dHRv, dHd, dHdv, dHld, dHrd, npts, dE,
                                    qidx ? dq : nullptr, zero_flag ? dz : nullptr, eta, eta0, dev_factor,
                                    convergence, max_iter, refine_iters, dTL, dst, dit, dws, ws, s);
  else
    rc = pf_transport_tdb_dev(n, nl, nr, L, nq, dHL, dHLv, dHR, dHRv, dHd, dHdv, dHld, dHrd, npts, dE,
                              qidx ? dq : nullptr, zero_flag ? dz : nullptr, eta, eta0, dev_factor, convergence,
                              max_iter, want_transr, dTL, dTR, dst, dit, dws, ws, s);
  if (rc != PF_SUCCESS) return rc;
  PF_CUDA(cudaMemcpyAsync(transl, dTL, b_E, cudaMemcpyDeviceToHost, s));
  if (want_transr) PF_CUDA(cudaMemcpyAsync(transr, dTR, b_E, cudaMemcpyDeviceToHost, s));
  PF_CUDA(cudaMemcpyAsync(status, dst, b_i, cudaMemcpyDeviceToHost, s));
  if (iters) PF_CUDA(cudaMemcpyAsync(iters, dit, 2 * b_i, cudaMemcpyDeviceToHost, s));
  PF_CUDA(cudaStreamSynchronize(s));
  int any = 0;
  for (int i = 0; i < npts; ++i) any |= status[i];
  if (any) {
    snprintf(g_err, sizeof(g_err), "pf: point status flags 0x%x (1 singular, 2 nan, 4 not converged)", any);
    return PF_ERR_POINT;
  }
  return PF_SUCCESS;
}
}  // namespace

extern "C" {

const char* pf_last_error(void) { return g_err; }

int pf_version(void) { return PF_ABI_VERSION; }

size_t pf_transport_tdb_workspace_size(int n, int nl, int nr, int npts) {
  if (check_dims(n, nl, nr, 1, 1, npts) != PF_SUCCESS) return 0;
  return workspace_bytes<double>(n, nl, nr, npts);
}

int pf_transport_tdb_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                         const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                         const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                         const int* zero_flag, double eta, double eta0, double dev_factor, double convergence,
                         int max_iter, int want_transr, double* transl, double* transr, int* status,
                         int* iters, void* work, size_t work_bytes, void* stream) {
  int rc = check_dims(n, nl, nr, L, nq, npts);
  if (rc != PF_SUCCESS) return rc;
  if (!E || !transl || !status || (want_transr && !transr))
    return set_err(PF_ERR_ARG, "pf: null energy/output pointer");
  if (!HL || !HLv || !HR || !HRv || !Hd || !Hld || !Hrd || (L > 1 && !Hdv))
    return set_err(PF_ERR_ARG, "pf: null block pointer");
  if (max_iter <= 0) return set_err(PF_ERR_ARG, "pf: max_iter must be positive");
  pf::System<double> sys = make_sys(n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd);
  pf::Points pts{npts, E, qidx, zero_flag};
  pf::Params P{eta, eta0, dev_factor, convergence, max_iter, want_transr};
  pf::Outputs out{transl, want_transr ? transr : nullptr, status, iters};
  return launch_transport<double>(sys, pts, P, out, work, work_bytes, (cudaStream_t)stream);
}

size_t pf_transport_tdb_mixed_workspace_size(int n, int nl, int nr, int L, int nq, int npts) {
  if (check_dims(n, nl, nr, L, nq, npts) != PF_SUCCESS) return 0;
  return mixed_workspace_bytes(n, nl, nr, L, nq, npts);
}

int pf_transport_tdb_mixed_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                               const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                               const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                               const int* zero_flag, double eta, double eta0, double dev_factor,
                               double convergence, int max_iter, int refine_iters, double* transl, int* status,
                               int* iters, void* work, size_t work_bytes, void* stream) {
  int rc = check_dims(n, nl, nr, L, nq, npts);
  if (rc != PF_SUCCESS) return rc;
  if (!E || !transl || !status) return set_err(PF_ERR_ARG, "pf: null energy/output pointer");
  if (!HL || !HLv || !HR || !HRv || !Hd || !Hld || !Hrd || (L > 1 && !Hdv))
    return set_err(PF_ERR_ARG, "pf: null block pointer");
  if (max_iter <= 0 || refine_iters < 0 || refine_iters > 16)
    return set_err(PF_ERR_ARG, "pf: max_iter must be positive and refine_iters in [0, 16]");
  if (npts == 0) return PF_SUCCESS;
  MixedLayout lay = make_mixed_layout(n, nl, nr, L, nq);
  DevInfo d = device_info();
  if (lay.smem > d.smem_optin) return set_err(PF_ERR_SIZE, "pf: working set exceeds shared memory");
  const int S = (lay.base.m + 31) / 32;
  const int grid = (S == 1) ? mixed_grid<1>(lay, npts) : mixed_grid<2>(lay, npts);
  if (grid <= 0) return set_err(PF_ERR_SIZE, "pf: kernel does not fit on the device");
  const size_t need = 256 + lay.blocks_d + lay.blocks_f + (size_t)grid * lay.per_cta;
  if (!work || work_bytes < need) return set_err(PF_ERR_ARG, "pf: workspace too small");
  cudaStream_t st = (cudaStream_t)stream;
  char* w = reinterpret_cast<char*>(work);
  int* queue = reinterpret_cast<int*>(w);
  char* p = w + 256;
  const double* src[8] = {HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd};
  dcx* dd[8];
  for (int i = 0; i < 8; ++i) {
    dd[i] = reinterpret_cast<dcx*>(p);
    p += (lay.cnt[i] * 16 + 255) & ~(size_t)255;
  }
  fcx* ff[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  for (int i = 2; i < 8; ++i) {
    ff[i] = reinterpret_cast<fcx*>(p);
    p += (lay.cnt[i] * 8 + 255) & ~(size_t)255;
  }
  char* scratch = p;
  for (int i = 0; i < 8; ++i) {
    if (lay.cnt[i] == 0) continue;
    const int blocks = (int)((lay.cnt[i] + 255) / 256 < 4096 ? (lay.cnt[i] + 255) / 256 : 4096);
    convert_blocks_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<const cx<double>*>(src[i]), dd[i],
                                                   i >= 2 ? ff[i] : nullptr, lay.cnt[i]);
  }
  PF_CUDA(cudaGetLastError());
  pf::MSys sys;
  sys.n = n;
  sys.nl = nl;
  sys.nr = nr;
  sys.L = L;
  sys.nq = nq;
  sys.HL = dd[0];
  sys.HLv = dd[1];
  sys.HR = dd[2];
  sys.HRv = dd[3];
  sys.Hd = dd[4];
  sys.Hdv = dd[5];
  sys.Hld = dd[6];
  sys.Hrd = dd[7];
  sys.fHR = ff[2];
  sys.fHd = ff[4];
  sys.fHdv = ff[5];
  sys.fHld = ff[6];
  sys.fHrd = ff[7];
  pf::Points pts{npts, E, qidx, zero_flag};
  pf::Params P{eta, eta0, dev_factor, convergence, max_iter, 0};
  pf::Outputs out{transl, nullptr, status, iters};
  PF_CUDA(cudaMemsetAsync(queue, 0, sizeof(int), st));
  if (S == 1)
    mixed_kernel<1><<<grid, kThreads, lay.smem, st>>>(sys, pts, P, refine_iters, out, lay, scratch, queue);
  else
    mixed_kernel<2><<<grid, kThreads, lay.smem, st>>>(sys, pts, P, refine_iters, out, lay, scratch, queue);
  PF_CUDA(cudaGetLastError());
  return PF_SUCCESS;
}

int pf_transport_tdb_mixed(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                           const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                           const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                           const int* zero_flag, double eta, double eta0, double dev_factor, double convergence,
                           int max_iter, int refine_iters, double* transl, int* status, int* iters) {
  return host_run(true, refine_iters, n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd, npts, E, qidx,
                  zero_flag, eta, eta0, dev_factor, convergence, max_iter, 0, transl, nullptr, status, iters);
}

int pf_transport_tdb(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv, const double* HR,
                     const double* HRv, const double* Hd, const double* Hdv, const double* Hld,
                     const double* Hrd, int npts, const double* E, const int* qidx, const int* zero_flag,
                     double eta, double eta0, double dev_factor, double convergence, int max_iter,
                     int want_transr, double* transl, double* transr, int* status, int* iters) {
  return host_run(false, 0, n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd, npts, E, qidx, zero_flag, eta,
                  eta0, dev_factor, convergence, max_iter, want_transr, transl, transr, status, iters);
}

}  // extern "C"
