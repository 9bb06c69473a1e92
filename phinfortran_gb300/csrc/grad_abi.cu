// extern "C" entry of the adjoint (gradient) of the transmission.
//
// pf_transport_tdb_grad_dev returns, for a batch of points with weights
// w_p, the forward T_L of every point and the accumulated sensitivities
//   M_B = sum_p w_p dT_p/dB   (dF = Re Tr[dB M_B], F = sum_p w_p T_p)
// for every device block B (Hd, Hdv) and the lead-device couplings
// (Hld, Hrd).  Chaining M_B to masses, springs or onsite energies is a
// sparse contraction done by the caller (phinfortran_gb300/gradients.py).
#include <cuda_runtime.h>
#include <stdio.h>

#include "../../include/phinfortran_gb300.h"
#include "adjoint.cuh"

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
#define GR_CUDA(call)                                  \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_err(e_, #call); \
  } while (0)

constexpr int kThreads = 256;

struct GLayout {
  int m, ld;
  size_t mat, smem, per_cta;
};

GLayout glayout(int n, int nl, int nr, int L) {
  GLayout g;
  g.m = n > nl ? n : nl;
  g.m = g.m > nr ? g.m : nr;
  g.ld = g.m | 1;
  g.mat = (size_t)g.ld * g.m;
  g.smem = pf::NSM * g.mat * 16 + 32 * sizeof(double) + 2 * (size_t)g.m * 16 + (size_t)g.m * 4 + 64 * 4;
  g.per_cta = ((size_t)pf::NG * g.mat * 16 + (3 * (size_t)(L + 2) + 2) * g.mat * 16 + 255) & ~(size_t)255;
  return g;
}

template <int S>
__global__ void __launch_bounds__(kThreads) grad_kernel(pf::System<double> sys, pf::Points pts, pf::Params P,
                                                        const double* weights, pf::Outputs out, pf::GradOut go,
                                                        GLayout lay, char* scratch, int* queue) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pf::Ctx<double> c;
  cx<double>* s = reinterpret_cast<cx<double>*>(smem_raw);
  for (int i = 0; i < pf::NSM; ++i) c.sm[i] = s + i * lay.mat;
  unsigned char* tail = reinterpret_cast<unsigned char*>(s + pf::NSM * lay.mat);
  c.red = reinterpret_cast<double*>(tail);
  c.iw.rowk = reinterpret_cast<cx<double>*>(tail + 32 * sizeof(double));
  c.iw.colk = c.iw.rowk + lay.m;
  int* ip = reinterpret_cast<int*>(c.iw.colk + lay.m);
  c.iw.perm = ip;
  c.iw.flag = ip + lay.m;
  cx<double>* g = reinterpret_cast<cx<double>*>(scratch + (size_t)blockIdx.x * lay.per_cta);
  for (int i = 0; i < pf::NG; ++i) c.gs[i] = g + i * lay.mat;
  c.ld = lay.ld;
  pf::GradSlabs sl;
  sl.mat = lay.mat;
  sl.lu = g + pf::NG * lay.mat;
  sl.xs = sl.lu + (size_t)(sys.L + 2) * lay.mat;
  sl.ys = sl.xs + (size_t)(sys.L + 2) * lay.mat;
  sl.k0 = sl.ys + (size_t)(sys.L + 2) * lay.mat;
  sl.k1 = sl.k0 + lay.mat;
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
    int st = pf::lead_pair<double, S>(c, sys, q, E, P, &itl, &itr);
    const double eps = E * P.eta + P.eta0;
    const cx<double> zD = pf::mk<double>(E, P.dev_factor * eps);
    const bool zero = pts.zero_flag && pts.zero_flag[p];
    const double w = (weights ? weights[p] : 1.0) * (zero ? 0.0 : 1.0);
    double tl = 0.0;
    st |= pf::adjoint_point<S>(c, sys, q, zD, w, sl, go, &tl);
    if (threadIdx.x == 0) {
      double a = tl;
      if (zero || a < 1.0e-60) a = 0.0;
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

int grad_grid(const GLayout& lay, int npts, int S) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (S == 1) {
    if (cudaFuncSetAttribute(grad_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.smem) !=
        cudaSuccess)
      return -1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grad_kernel<1>, kThreads, lay.smem) != cudaSuccess)
      return -1;
  } else {
    if (cudaFuncSetAttribute(grad_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.smem) !=
        cudaSuccess)
      return -1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grad_kernel<2>, kThreads, lay.smem) != cudaSuccess)
      return -1;
  }
  if (per_sm < 1) return -1;
  const int g = sms * per_sm;
  return g < npts ? g : npts;
}

// lead mirror flags (same rule as the transport entry)
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

}  // namespace

extern "C" {

const char* pf_grad_last_error(void) { return g_err; }

size_t pf_transport_tdb_grad_workspace_size(int n, int nl, int nr, int L, int nq, int npts) {
  if (n <= 0 || nl <= 0 || nr <= 0 || L <= 0 || nq <= 0 || npts < 0) return 0;
  if (n > PF_NMAX_RESIDENT || nl > PF_NMAX_RESIDENT || nr > PF_NMAX_RESIDENT) return 0;
  GLayout lay = glayout(n, nl, nr, L);
  const int S = (lay.m + 31) / 32;
  const int g = grad_grid(lay, npts > 0 ? npts : 1, S);
  if (g <= 0) return 0;
  return 256 + (((size_t)nq * 4 + 255) & ~(size_t)255) + (size_t)g * lay.per_cta;
}

int pf_transport_tdb_grad_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                              const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                              const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                              const int* zero_flag, const double* weights, double eta, double eta0,
                              double dev_factor, double convergence, int max_iter, double* transl, int* status,
                              int* iters, double* gHd, double* gHdv, double* gHld, double* gHrd, void* work,
                              size_t work_bytes, void* stream) {
  if (n <= 0 || nl <= 0 || nr <= 0 || L <= 0 || nq <= 0 || npts < 0)
    return set_err(PF_ERR_ARG, "pf_grad: dimensions must be positive");
  if (n > PF_NMAX_RESIDENT || nl > PF_NMAX_RESIDENT || nr > PF_NMAX_RESIDENT)
    return set_err(PF_ERR_SIZE, "pf_grad: block size exceeds the resident kernel limit");
  if (!E || !transl || !status || !gHd || !gHld || !gHrd || (L > 1 && !gHdv))
    return set_err(PF_ERR_ARG, "pf_grad: null pointer");
  if (!HL || !HLv || !HR || !HRv || !Hd || !Hld || !Hrd || (L > 1 && !Hdv))
    return set_err(PF_ERR_ARG, "pf_grad: null block pointer");
  if (max_iter <= 0) return set_err(PF_ERR_ARG, "pf_grad: max_iter must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  // zero the accumulators
  GR_CUDA(cudaMemsetAsync(gHd, 0, (size_t)nq * L * n * n * 16, st));
  if (L > 1) GR_CUDA(cudaMemsetAsync(gHdv, 0, (size_t)nq * (L - 1) * n * n * 16, st));
  GR_CUDA(cudaMemsetAsync(gHld, 0, (size_t)nq * n * nl * 16, st));
  GR_CUDA(cudaMemsetAsync(gHrd, 0, (size_t)nq * n * nr * 16, st));
  if (npts == 0) return PF_SUCCESS;
  GLayout lay = glayout(n, nl, nr, L);
  const int S = (lay.m + 31) / 32;
  const int grid = grad_grid(lay, npts, S);
  if (grid <= 0) return set_err(PF_ERR_SIZE, "pf_grad: kernel does not fit on the device");
  const size_t mir = ((size_t)nq * 4 + 255) & ~(size_t)255;
  if (!work || work_bytes < 256 + mir + (size_t)grid * lay.per_cta)
    return set_err(PF_ERR_ARG, "pf_grad: workspace too small");
  int* queue = reinterpret_cast<int*>(work);
  int* mirror = reinterpret_cast<int*>(reinterpret_cast<char*>(work) + 256);
  char* scratch = reinterpret_cast<char*>(work) + 256 + mir;
  GR_CUDA(cudaMemsetAsync(queue, 0, sizeof(int), st));
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
  pf::Params P{nullptr, eta, eta0, dev_factor, convergence, max_iter, 0};
  if (nl == nr) {
    mirror_kernel<<<nq, 256, 0, st>>>(HL, HLv, HR, HRv, 2 * nl * nl, nq, mirror);
    P.lead_mirror = mirror;
  }
  pf::Outputs out{transl, nullptr, status, iters};
  pf::GradOut go;
  go.gHd = reinterpret_cast<cx<double>*>(gHd);
  go.gHdv = reinterpret_cast<cx<double>*>(gHdv);
  go.gHld = reinterpret_cast<cx<double>*>(gHld);
  go.gHrd = reinterpret_cast<cx<double>*>(gHrd);
  if (S == 1)
    grad_kernel<1><<<grid, kThreads, lay.smem, st>>>(sys, pts, P, weights, out, go, lay, scratch, queue);
  else
    grad_kernel<2><<<grid, kThreads, lay.smem, st>>>(sys, pts, P, weights, out, go, lay, scratch, queue);
  GR_CUDA(cudaGetLastError());
  return PF_SUCCESS;
}

}  // extern "C"
