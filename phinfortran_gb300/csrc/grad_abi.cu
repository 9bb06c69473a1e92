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
#include "grad_impl.cuh"

using pf::cx;
using pfgrad::GLayout;
using pfgrad::glayout;

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

// bytes of the double-float copy of the blocks (0 for FP64)
size_t df64_blocks_bytes(int n, int nl, int nr, int L, int nq, int arith) {
  if (arith != PF_ARITH_DF64) return 0;
  const size_t c = (size_t)nq * (2 * (size_t)nl * nl + 2 * (size_t)nr * nr + (size_t)L * n * n +
                                 (size_t)(L > 1 ? L - 1 : 0) * n * n + (size_t)nl * n + (size_t)nr * n);
  return ((c * 16) + 255) & ~(size_t)255;
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

size_t pf_transport_tdb_grad_workspace_size(int n, int nl, int nr, int L, int nq, int npts, int ckpt,
                                            int arith) {
  if (n <= 0 || nl <= 0 || nr <= 0 || L <= 0 || nq <= 0 || npts < 0 || ckpt < 0) return 0;
  if (arith != PF_ARITH_FP64 && arith != PF_ARITH_DF64) return 0;
  if (n > PF_NMAX_RESIDENT || nl > PF_NMAX_RESIDENT || nr > PF_NMAX_RESIDENT) return 0;
  GLayout lay = glayout(n, nl, nr, L, ckpt);
  const int np = npts > 0 ? npts : 1;
  const int g = arith == PF_ARITH_FP64 ? pfgrad::grid_fp64(lay, np) : pfgrad::grid_df64(lay, np);
  if (g <= 0) return 0;
  return 256 + (((size_t)nq * 4 + 255) & ~(size_t)255) + (size_t)g * lay.per_cta + df64_blocks_bytes(n, nl, nr, L, nq, arith);
}

int pf_transport_tdb_grad_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                              const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                              const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                              const int* zero_flag, const double* weights, double eta, double eta0,
                              double dev_factor, double convergence, int max_iter, int ckpt, int arith,
                              double* transl, int* status,
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
  if (ckpt < 0) return set_err(PF_ERR_ARG, "pf_grad: checkpoint interval must be >= 0");
  if (arith != PF_ARITH_FP64 && arith != PF_ARITH_DF64) return set_err(PF_ERR_ARG, "pf_grad: unknown arithmetic");
  cudaStream_t st = (cudaStream_t)stream;
  // zero the accumulators
  GR_CUDA(cudaMemsetAsync(gHd, 0, (size_t)nq * L * n * n * 16, st));
  if (L > 1) GR_CUDA(cudaMemsetAsync(gHdv, 0, (size_t)nq * (L - 1) * n * n * 16, st));
  GR_CUDA(cudaMemsetAsync(gHld, 0, (size_t)nq * n * nl * 16, st));
  GR_CUDA(cudaMemsetAsync(gHrd, 0, (size_t)nq * n * nr * 16, st));
  if (npts == 0) return PF_SUCCESS;
  GLayout lay = glayout(n, nl, nr, L, ckpt);
  const int grid = arith == PF_ARITH_FP64 ? pfgrad::grid_fp64(lay, npts) : pfgrad::grid_df64(lay, npts);
  if (grid <= 0) return set_err(PF_ERR_SIZE, "pf_grad: kernel does not fit on the device");
  const size_t mir = ((size_t)nq * 4 + 255) & ~(size_t)255;
  const size_t dfb = df64_blocks_bytes(n, nl, nr, L, nq, arith);
  if (!work || work_bytes < 256 + mir + (size_t)grid * lay.per_cta + dfb)
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
  if (arith == PF_ARITH_FP64)
    pfgrad::launch_fp64(grid, lay, sys, pts, P, weights, out, go, scratch, queue, st);
  else
    pfgrad::launch_df64(grid, lay, sys, reinterpret_cast<pf::df64*>(scratch + (size_t)grid * lay.per_cta), pts, P,
                        weights, out, go, scratch, queue, st);
  GR_CUDA(cudaGetLastError());
  return PF_SUCCESS;
}

}  // extern "C"
