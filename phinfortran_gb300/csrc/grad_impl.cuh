// Gradient kernel shared by the FP64 and double-float translation units.
#pragma once
#include <cuda_runtime.h>

#include "adjoint.cuh"

namespace pfgrad {

using pf::cx;

constexpr int kThreads = 512;  // one CTA per SM (shared memory): 16 warps per point

struct GLayout {
  int m, ld;
  int seg;   // checkpoint interval (1: every layer kept, no recomputation)
  int nseg;  // checkpoints
  size_t mat, smem, per_cta;
};

// ckpt = 0 picks ceil(sqrt(L + 2)); ckpt = 1 keeps every layer.
inline GLayout glayout(int n, int nl, int nr, int L, int ckpt) {
  GLayout g;
  g.m = n > nl ? n : nl;
  g.m = g.m > nr ? g.m : nr;
  g.ld = g.m | 1;
  g.mat = (size_t)g.ld * g.m;
  g.smem = pf::NSM * g.mat * 16 + 32 * sizeof(double) + 2 * (size_t)g.m * 16 + (size_t)g.m * 4 + 64 * 4;
  int seg = ckpt;
  if (seg <= 0) {
    seg = 1;
    while (seg * seg < L + 2) ++seg;
  }
  if (seg > L + 2) seg = L + 2;
  g.seg = seg;
  g.nseg = (L + 2 + seg - 1) / seg;
  const size_t slabs = (seg == 1) ? 3 * (size_t)(L + 2) + 2 : 2 * (size_t)g.nseg + 2 * (size_t)seg + 8;
  g.per_cta = ((size_t)pf::NG * g.mat * 16 + slabs * g.mat * 16 + 255) & ~(size_t)255;
  return g;
}

template <typename R, int S, bool CK>
__global__ void __launch_bounds__(kThreads) grad_kernel(pf::System<R> sys, pf::Points pts, pf::Params P,
                                                        const double* weights, pf::Outputs out, pf::GradOut go,
                                                        GLayout lay, char* scratch, int* queue) {
  static_assert(sizeof(cx<R>) == 16, "slot sizes assume 16-byte complex elements");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pf::Ctx<R> c;
  cx<R>* s = reinterpret_cast<cx<R>*>(smem_raw);
  for (int i = 0; i < pf::NSM; ++i) c.sm[i] = s + i * lay.mat;
  unsigned char* tail = reinterpret_cast<unsigned char*>(s + pf::NSM * lay.mat);
  c.red = reinterpret_cast<double*>(tail);
  c.iw.rowk = reinterpret_cast<cx<R>*>(tail + 32 * sizeof(double));
  c.iw.colk = c.iw.rowk + lay.m;
  int* ip = reinterpret_cast<int*>(c.iw.colk + lay.m);
  c.iw.perm = ip;
  c.iw.flag = ip + lay.m;
  cx<R>* g = reinterpret_cast<cx<R>*>(scratch + (size_t)blockIdx.x * lay.per_cta);
  for (int i = 0; i < pf::NG; ++i) c.gs[i] = g + i * lay.mat;
  c.ld = lay.ld;
  pf::GradSlabs<R> sl;
  sl.mat = lay.mat;
  sl.lu = g + pf::NG * lay.mat;
  sl.xs = sl.lu + (size_t)(sys.L + 2) * lay.mat;
  sl.ys = sl.xs + (size_t)(sys.L + 2) * lay.mat;
  sl.k0 = sl.ys + (size_t)(sys.L + 2) * lay.mat;
  sl.k1 = sl.k0 + lay.mat;
  pf::CkptSlabs<R> ck;
  ck.mat = lay.mat;
  ck.seg = lay.seg;
  ck.ckg = g + pf::NG * lay.mat;
  ck.cky = ck.ckg + (size_t)lay.nseg * lay.mat;
  ck.segg = ck.cky + (size_t)lay.nseg * lay.mat;
  ck.segy = ck.segg + (size_t)lay.seg * lay.mat;
  ck.pg = ck.segy + (size_t)lay.seg * lay.mat;
  ck.py = ck.pg + lay.mat;
  ck.pG0 = ck.py + lay.mat;
  ck.W = ck.pG0 + lay.mat;
  ck.xa = ck.W + lay.mat;
  ck.xb = ck.xa + lay.mat;
  ck.k0 = ck.xb + lay.mat;
  ck.k1 = ck.k0 + lay.mat;
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
    const bool zero = pts.zero_flag && pts.zero_flag[p];
    const double w = (weights ? weights[p] : 1.0) * (zero ? 0.0 : 1.0);
    double tl = 0.0;
    if (CK)
      st |= pf::adjoint_point_ckpt<R, S>(c, sys, q, zD, w, ck, go, &tl);
    else
      st |= pf::adjoint_point<R, S>(c, sys, q, zD, w, sl, go, &tl);
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

template <typename R, int S, bool CK>
int grad_grid_t(const GLayout& lay, int npts) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaFuncSetAttribute(grad_kernel<R, S, CK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.smem) !=
      cudaSuccess)
    return -1;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grad_kernel<R, S, CK>, kThreads, lay.smem) !=
      cudaSuccess)
    return -1;
  if (per_sm < 1) return -1;
  const int g = sms * per_sm;
  return g < npts ? g : npts;
}

template <typename R>
int grad_grid_r(const GLayout& lay, int npts) {
  const int S = (lay.m + 31) / 32;
  const bool ck = lay.seg > 1;
  if (S == 1) return ck ? grad_grid_t<R, 1, true>(lay, npts) : grad_grid_t<R, 1, false>(lay, npts);
  return ck ? grad_grid_t<R, 2, true>(lay, npts) : grad_grid_t<R, 2, false>(lay, npts);
}

template <typename R>
void grad_launch_r(int grid, const GLayout& lay, const pf::System<R>& sys, const pf::Points& pts,
                   const pf::Params& P, const double* weights, const pf::Outputs& out, const pf::GradOut& go,
                   char* scratch, int* queue, cudaStream_t st) {
  const int S = (lay.m + 31) / 32;
  const bool ck = lay.seg > 1;
  if (S == 1 && !ck)
    grad_kernel<R, 1, false><<<grid, kThreads, lay.smem, st>>>(sys, pts, P, weights, out, go, lay, scratch, queue);
  else if (S == 1)
    grad_kernel<R, 1, true><<<grid, kThreads, lay.smem, st>>>(sys, pts, P, weights, out, go, lay, scratch, queue);
  else if (!ck)
    grad_kernel<R, 2, false><<<grid, kThreads, lay.smem, st>>>(sys, pts, P, weights, out, go, lay, scratch, queue);
  else
    grad_kernel<R, 2, true><<<grid, kThreads, lay.smem, st>>>(sys, pts, P, weights, out, go, lay, scratch, queue);
}


// Per-arithmetic entry points (grad_fp64.cu, grad_df64.cu).
int grid_fp64(const GLayout& lay, int npts);
int grid_df64(const GLayout& lay, int npts);
void launch_fp64(int grid, const GLayout& lay, const pf::System<double>& sys, const pf::Points& pts,
                 const pf::Params& P, const double* weights, const pf::Outputs& out, const pf::GradOut& go,
                 char* scratch, int* queue, cudaStream_t st);
// converts the FP64 blocks of `sys` into `dst` (double-float) and launches
void launch_df64(int grid, const GLayout& lay, const pf::System<double>& sys, pf::df64* dst, const pf::Points& pts,
                 const pf::Params& P, const double* weights, const pf::Outputs& out, const pf::GradOut& go,
                 char* scratch, int* queue, cudaStream_t st);

}  // namespace pfgrad
