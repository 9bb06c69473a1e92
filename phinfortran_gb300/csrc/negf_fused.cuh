// The mixed pipeline's layout and the fused kernel of cross-sections above
// 32 (a CTA of kMixedThreads per point: both lead decimations, the FP32
// block LU, the double-float refinement and the Caroli trace in one
// launch).  The fused kernel is compiled in its own translation unit
// (negf_fused.cu, which defines PF_FUSED_S); negf_mixed.cu reaches it
// through fused_per_sm and fused_launch.
#pragma once
#include "negf_common.cuh"
#include "warp_engine.cuh"

using pf::dcx;
using pf::fcx;

namespace pfn {

constexpr int kMixedThreads = 512;  // fused mixed kernel: one CTA per SM, 16 warps per point

struct MixedLayout {
  Layout base;     // smem slots are df64-sized (16 B per complex)
  size_t smem;
  size_t smem_leads;  // the leads kernel needs only the NSM decimation slots
  size_t per_cta;  // bytes of per-CTA scratch
  size_t blocks_d, blocks_f;  // bytes of converted block copies (per call)
  size_t cnt[8];   // complex elements per block family (all q)
  size_t ell_rows[7];  // ELL rows: Hd, Hdv, Hdv^H, Hld, Hld^H, Hrd, Hrd^H
  size_t ell_bytes;
};

inline MixedLayout make_mixed_layout(int n, int nl, int nr, int L, int nq) {
  MixedLayout m;
  m.base = make_layout<double>(n, nl, nr);
  const size_t mat = m.base.mat;
  const size_t tail = 32 * sizeof(double) + 2 * (size_t)m.base.m * 16 + (size_t)m.base.m * sizeof(int) +
                      64 * sizeof(int);
  m.smem = pf::NSM_M * mat * 16 + tail;
  m.smem_leads = pf::NSM * mat * 16 + tail;
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
  const size_t er[7] = {(size_t)nq * L * n, (size_t)nq * (L > 1 ? L - 1 : 0) * n,
                        (size_t)nq * (L > 1 ? L - 1 : 0) * n, (size_t)nq * nl, (size_t)nq * n, (size_t)nq * nr,
                        (size_t)nq * n};
  size_t eb = 256;  // overflow flag
  for (int i = 0; i < 7; ++i) {
    m.ell_rows[i] = er[i];
    eb += ((er[i] * pf::PF_ELL_K * 4 + 255) & ~(size_t)255) + ((er[i] * pf::PF_ELL_K * 16 + 255) & ~(size_t)255);
  }
  m.ell_bytes = eb + (((size_t)nq * sizeof(int) + 255) & ~(size_t)255);  // + lead mirror flags
  return m;
}


// Occupancy (CTAs per SM) of the fused kernel with `smem` dynamic shared
// memory (sets the kernel's shared-memory attribute; 0 on error) and its
// launch.  Only tiles of 64 (S = 2) exist: blocks up to 32 never reach
// the fused kernel, so S = 1 reports no occupancy.
int fused_per_sm_2(size_t smem);
cudaError_t fused_launch_2(int grid, size_t smem, cudaStream_t st, const pf::MSys& sys, const pf::Points& pts,
                           const pf::Params& P, int nref, const pf::Outputs& out, const MixedLayout& lay,
                           char* scratch, int* queue);
inline int fused_per_sm(int S, size_t smem) { return S == 2 ? fused_per_sm_2(smem) : 0; }
inline cudaError_t fused_launch(int S, int grid, size_t smem, cudaStream_t st, const pf::MSys& sys,
                                const pf::Points& pts, const pf::Params& P, int nref, const pf::Outputs& out,
                                const MixedLayout& lay, char* scratch, int* queue) {
  return S == 2 ? fused_launch_2(grid, smem, st, sys, pts, P, nref, out, lay, scratch, queue)
                : cudaErrorInvalidValue;
}

}  // namespace pfn

#ifdef PF_FUSED_S
namespace pfn {
namespace {
template <int S>
__global__ void __launch_bounds__(kMixedThreads) mixed_kernel(pf::MSys sys, pf::Points pts, pf::Params P, int nref,
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
    // the first sweep always; later ones while the last correction of X_0
    // was above PF_REFINE_TOL
    for (int k = 0; k < nref; ++k)
      if (!pf::mixed_refine<S>(c, sys, q, zL, zD)) break;
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


}  // namespace

#define PF_FUSED_CAT2(a, b) a##b
#define PF_FUSED_CAT(a, b) PF_FUSED_CAT2(a, b)

int PF_FUSED_CAT(fused_per_sm_, PF_FUSED_S)(size_t smem) {
  auto k = mixed_kernel<PF_FUSED_S>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kMixedThreads, smem) != cudaSuccess) return 0;
  return per_sm;
}

cudaError_t PF_FUSED_CAT(fused_launch_, PF_FUSED_S)(int grid, size_t smem, cudaStream_t st, const pf::MSys& sys,
                                                    const pf::Points& pts, const pf::Params& P, int nref,
                                                    const pf::Outputs& out, const MixedLayout& lay, char* scratch,
                                                    int* queue) {
  mixed_kernel<PF_FUSED_S><<<grid, kMixedThreads, smem, st>>>(sys, pts, P, nref, out, lay, scratch, queue);
  return cudaGetLastError();
}

}  // namespace pfn
#endif
