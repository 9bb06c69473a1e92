// Two-probe Landauer conductance on the GPU.
//
// Reference: examples/negf/si-si/condt.py:14-30, the post-processing that
// turns T(omega) into a thermal conductance:
//   sigma(T) = 1/A * 1/(2 pi) * trapz( hbar w * df/dT * T(w), w ),
//   df/dT = e^x/(e^x-1)^2 * hbar w/(kB T^2),  x = hbar w/(kB T),
// evaluated for several temperatures at once with one CTA per temperature
// (block reduction of the trapezoid sum in FP64).
#include <cuda_runtime.h>
#include <stdio.h>

#include "../../include/phinfortran_gb300.h"

namespace {

thread_local char g_err[512] = "";

__global__ void condt_kernel(int ne, const double* w, const double* tr, const double* temps, double area,
                             double* out) {
  const double kb = 1.380649e-23, hbar = 1.0545718e-34, pi = 3.141592653589793238;
  const double T = temps[blockIdx.x];
  double acc = 0.0;
  for (int i = threadIdx.x; i < ne - 1; i += blockDim.x) {
    double itd[2];
    for (int s = 0; s < 2; ++s) {
      const double wi = w[i + s];
      const double expf = exp(hbar * wi / kb / T);
      const double dfdw = expf / ((expf - 1.0) * (expf - 1.0)) * hbar * wi / kb / (T * T);
      itd[s] = 1.0 / area / 2.0 / pi * (hbar * wi * dfdw * tr[i + s]);
    }
    acc += (itd[0] + itd[1]) * 0.5 * (w[i + 1] - w[i]);
  }
  __shared__ double red[1024];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

}  // namespace

extern "C" {

const char* pf_cond_last_error(void) { return g_err; }

int pf_landauer_conductance(int ne, const double* omega, const double* trans, int ntemp, const double* temps,
                            double area, double* sigma) {
  if (ne < 2 || ntemp < 1 || !omega || !trans || !temps || !sigma || !(area > 0.0)) {
    snprintf(g_err, sizeof(g_err), "pf_landauer_conductance: need ne >= 2, ntemp >= 1, area > 0, non-null arrays");
    return PF_ERR_ARG;
  }
  double *dw = nullptr, *dt = nullptr, *dT = nullptr, *dout = nullptr;
  cudaError_t e = cudaMalloc(&dw, (size_t)ne * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dt, (size_t)ne * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dT, (size_t)ntemp * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dout, (size_t)ntemp * 8);
  if (e == cudaSuccess) e = cudaMemcpy(dw, omega, (size_t)ne * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dt, trans, (size_t)ne * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dT, temps, (size_t)ntemp * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    condt_kernel<<<ntemp, 256>>>(ne, dw, dt, dT, area, dout);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(sigma, dout, (size_t)ntemp * 8, cudaMemcpyDeviceToHost);
  cudaFree(dw);
  cudaFree(dt);
  cudaFree(dT);
  cudaFree(dout);
  if (e != cudaSuccess) {
    snprintf(g_err, sizeof(g_err), "pf_landauer_conductance: %s", cudaGetErrorString(e));
    return PF_ERR_CUDA;
  }
  return PF_SUCCESS;
}

}  // extern "C"
