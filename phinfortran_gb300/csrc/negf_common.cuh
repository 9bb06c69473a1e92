// Pieces shared by the two translation units of the tdb transport entries
// (negf_abi.cu: the FP64 path, the host-pointer and allocation-free entries;
// negf_mixed.cu: the mixed-precision pipeline): the error buffer behind
// pf_last_error, the scratch layout of the CTA-level kernels, the lead
// mirror test and the size checks.  Everything but the error buffer is
// internal to each unit.
#pragma once
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include "../../include/phinfortran_gb300.h"
#include "transport.cuh"

using pf::cx;

// message of the last error of the tdb entries (defined in negf_abi.cu)
extern thread_local char pf_negf_err[512];

namespace pfn {

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

}  // namespace pfn

namespace {

int set_err(int code, const char* msg) {
  snprintf(pf_negf_err, sizeof(pf_negf_err), "%s", msg);
  return code;
}
int cuda_err(cudaError_t e, const char* where) {
  snprintf(pf_negf_err, sizeof(pf_negf_err), "%s: %s", where, cudaGetErrorString(e));
  return PF_ERR_CUDA;
}

#define PF_CUDA(call)                               \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return cuda_err(e_, #call); \
  } while (0)

constexpr int kThreads = 256;

using pfn::Layout;
using pfn::make_layout;



// mirror[q] = 1 when the right lead blocks equal the left ones bitwise.
__global__ void lead_mirror_kernel(const double* HL, const double* HLv, const double* HR, const double* HRv,
                                   int m2, int nq, int* mirror) {
  // m2 = 2 * nl * nl doubles per block; one CTA per q
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


int check_dims(int n, int nl, int nr, int L, int nq, int npts) {
  if (n <= 0 || nl <= 0 || nr <= 0 || L <= 0 || nq <= 0 || npts < 0)
    return set_err(PF_ERR_ARG, "pf: dimensions must be positive");
  if (n > PF_NMAX_RESIDENT || nl > PF_NMAX_RESIDENT || nr > PF_NMAX_RESIDENT)
    return set_err(PF_ERR_SIZE, "pf: block size exceeds the shared-memory resident kernel limit");
  return PF_SUCCESS;
}

}  // namespace
