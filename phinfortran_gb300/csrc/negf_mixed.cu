// Mixed-precision tdb transport (pf_transport_tdb_mixed_dev and its
// variants): FP64-grade lead decimations (block products on the tensor
// cores for blocks up to 32), FP32 block LU of the device, double-float
// refinement and Caroli trace.  The host-pointer entry
// pf_transport_tdb_mixed is in negf_abi.cu.
#include "negf_fused.cuh"

namespace {
// ===========================================================================
// Mixed-precision path
// ===========================================================================

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

// ELL copy of `count` blocks (rows x cols each, column-major).  With
// `ct` the ELL describes the conjugate transpose (rows of M^H = columns of M).
// One thread per output row; rows with more than K nonzeros set *overflow.
__global__ void build_ell_kernel(const dcx* M, int rows, int cols, int count, int ct, int K, int* col_out,
                                 dcx* val_out, int* overflow) {
  const int orows = ct ? cols : rows, ocols = ct ? rows : cols;
  const size_t total = (size_t)count * orows;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const size_t b = t / orows;
    const int r = (int)(t % orows);
    const dcx* Mb = M + b * (size_t)rows * cols;
    int k = 0;
    for (int c = 0; c < ocols; ++c) {
      dcx v = ct ? Mb[c + (size_t)r * rows] : Mb[r + (size_t)c * rows];
      if (ct) v = pf::cconj(v);
      const bool nz = v.x.hi != 0.f || v.x.lo != 0.f || v.y.hi != 0.f || v.y.lo != 0.f;
      if (!nz) continue;
      if (k < K) {
        const size_t at = pf::ell_at(b, K, orows, r, k);
        col_out[at] = c;
        val_out[at] = v;
      } else {
        atomicOr(overflow, 1);
      }
      ++k;
    }
    for (; k < K; ++k) col_out[pf::ell_at(b, K, orows, r, k)] = -1;
  }
}

using pfn::MixedLayout;
using pfn::make_mixed_layout;
using pfn::kMixedThreads;

// ---------------------------------------------------------------------------
// Mixed path, cross-sections <= 32: leads kernel (CTA per point) + layer
// kernel (warp per point).
// ---------------------------------------------------------------------------
constexpr int kWarpsPerCta = 4;
constexpr int kLayerCtasPerSm = 3;  // 12 warps per SM: 2 x 8.5 KB shared buffers and <= 170 registers a thread

// Copy an (m x m) df64/FP32 matrix from scratch (ld) into a padded 32x32
// per-point block (ld 32); `ident` puts ones on the padded diagonal.
template <typename T>
__device__ void pad_store(T* dst, const T* src, int ld, int m, bool ident) {
  for (int i = threadIdx.x; i < pf::wp::NW * pf::wp::NW; i += blockDim.x) {
    const int r = i % pf::wp::NW, c = i / pf::wp::NW;
    T v;
    v.x = decltype(v.x)(0.f, 0.f);
    v.y = decltype(v.y)(0.f, 0.f);
    if (r < m && c < m) v = src[r + c * ld];
    dst[i] = v;
  }
}
__device__ void pad_store_f(fcx* dst, const fcx* src, int ld, int m, bool ident) {
  for (int i = threadIdx.x; i < pf::wp::NW * pf::wp::NW; i += blockDim.x) {
    const int r = i % pf::wp::NW, c = i / pf::wp::NW;
    fcx v = pf::mk<float>(0.f, 0.f);
    if (r < m && c < m)
      v = src[r + c * ld];
    else if (ident && r == c)
      v = pf::mk<float>(1.f, 0.f);
    dst[i] = v;
  }
}

template <int S>
__global__ void __launch_bounds__(kThreads) leads_kernel(pf::MSys sys, pf::Points pts, pf::Params P,
                                                         pf::Outputs out, MixedLayout lay, size_t per_cta,
                                                         char* scratch, pf::wp::LeadOut lo, int* lead_status,
                                                         int* queue) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pf::MCtx c;
  const size_t mat = lay.base.mat;
  dcx* s = reinterpret_cast<dcx*>(smem_raw);
  for (int i = 0; i < pf::NSM_M; ++i) c.sm[i] = i < pf::NSM ? s + i * mat : nullptr;
  unsigned char* tail = reinterpret_cast<unsigned char*>(s + pf::NSM * mat);
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
  char* base = scratch + (size_t)blockIdx.x * per_cta;
  dcx* g = reinterpret_cast<dcx*>(base);
  for (int i = 0; i < pf::NGM; ++i) c.gs[i] = g + i * mat;
  // lu/fsr of the CTA scratch hold g_0 and Sigma_R before they are padded out
  c.xv = g + pf::NGM * mat;
  c.lu = reinterpret_cast<fcx*>(c.xv);
  c.yv = c.lu + mat;
  c.fsr = c.yv + mat;
  c.ld = lay.base.ld;
  c.mat = mat;
  __shared__ int s_p;
  const size_t B = (size_t)pf::wp::NW * pf::wp::NW;
  for (;;) {
    if (threadIdx.x == 0) s_p = atomicAdd(queue, 1);
    __syncthreads();
    const int p = s_p;
    __syncthreads();
    if (p >= pts.npts) break;
    const int q = pts.qidx ? pts.qidx[p] : 0;
    int itl = 0, itr = 0;
    const int st = pf::mixed_leads<S>(c, sys, q, pts.E[p], P, &itl, &itr);
    pad_store_f(lo.g0 + p * B, c.lu, c.ld, sys.nl, true);
    pad_store_f(lo.fsr + p * B, c.fsr, c.ld, sys.nr, false);
    pad_store(lo.esl + p * B, c.gs[pf::M_ESL], c.ld, sys.nl, false);
    pad_store(lo.sr + p * B, c.gs[pf::M_SR], c.ld, sys.nr, false);
    pad_store(lo.gml + p * B, c.gs[pf::M_GML], c.ld, sys.nl, false);
    pad_store(lo.gmr + p * B, c.gs[pf::M_GMR], c.ld, sys.nr, false);
    if (threadIdx.x == 0) {
      lead_status[p] = st;
      if (out.iters) {
        out.iters[2 * p] = itl;
        out.iters[2 * p + 1] = itr;
      }
    }
    __syncthreads();
  }
}


// Leads kernel of the FP64 lead arithmetic (blocks up to 32): the same work
// as leads_kernel<1>, the decimations' block products on the tensor cores
// (tc_small.cuh).  One CTA per SM: it holds all 512 TMEM columns (the
// dynamic shared memory requested keeps a second CTA off the SM).  With
// gs_smem the four working matrices of the decimation (e1, es and the two
// products W2, W3) are in shared memory instead of the CTA's global
// scratch: three after the tensor-core tiles, W3 in SM3 (the decimation's
// inverse uses SM3 as its second buffer only while W3 is dead).
constexpr int kLeadsTcShared = 3;  // M_E1, M_ES, M_W2 (M_W3 in SM3)
static_assert(kThreads == pf::tc::kSmallThreads, "small_zgemm is written for the leads CTA size");
__global__ void __launch_bounds__(kThreads, 1) leads_tc_kernel(pf::MSys sys, pf::Points pts, pf::Params P,
                                                         pf::Outputs out, MixedLayout lay, size_t per_cta,
                                                         char* scratch, pf::wp::LeadOut lo, int* lead_status,
                                                         int* queue, int gs_smem) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int S = 1;
  pf::MCtx c;
  const size_t mat = lay.base.mat;
  dcx* s = reinterpret_cast<dcx*>(smem_raw);
  for (int i = 0; i < pf::NSM_M; ++i) c.sm[i] = i < pf::NSM ? s + i * mat : nullptr;
  unsigned char* tail = reinterpret_cast<unsigned char*>(s + pf::NSM * mat);
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
  char* base = scratch + (size_t)blockIdx.x * per_cta;
  dcx* g = reinterpret_cast<dcx*>(base);
  for (int i = 0; i < pf::NGM; ++i) c.gs[i] = g + i * mat;
  // lu/fsr of the CTA scratch hold g_0 and Sigma_R before they are padded out
  c.xv = g + pf::NGM * mat;
  c.lu = reinterpret_cast<fcx*>(c.xv);
  c.yv = c.lu + mat;
  c.fsr = c.yv + mat;
  c.ld = lay.base.ld;
  c.mat = mat;
  __shared__ int s_p;
  __shared__ int s_tc_abort;
  const size_t B = (size_t)pf::wp::NW * pf::wp::NW;
  // tensor-core tiles after the decimation slots, 1024-aligned
  unsigned char* tiles = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + lay.smem_leads + 1023) & ~(uintptr_t)1023);
  if (gs_smem) {
    static_assert(pf::M_E1 == 0 && pf::M_ES == 1 && pf::M_W2 == 2 && pf::M_W3 == 3, "decimation slots first");
    dcx* gsm = reinterpret_cast<dcx*>(tiles + pf::tc::kSmallSmem);
    for (int i = 0; i < kLeadsTcShared; ++i) c.gs[i] = gsm + i * mat;
    c.gs[pf::M_W3] = c.sm[3];
  }
  pf::tc::SmallTC tcx;
  pf::tc::small_init(tcx, tiles, &s_tc_abort);
  for (;;) {
    if (threadIdx.x == 0) s_p = atomicAdd(queue, 1);
    __syncthreads();
    const int p = s_p;
    __syncthreads();
    if (p >= pts.npts) break;
    const int q = pts.qidx ? pts.qidx[p] : 0;
    int itl = 0, itr = 0;
    const int st = pf::mixed_leads<S>(c, sys, q, pts.E[p], P, &itl, &itr, &tcx);
    pad_store_f(lo.g0 + p * B, c.lu, c.ld, sys.nl, true);
    pad_store_f(lo.fsr + p * B, c.fsr, c.ld, sys.nr, false);
    pad_store(lo.esl + p * B, c.gs[pf::M_ESL], c.ld, sys.nl, false);
    pad_store(lo.sr + p * B, c.gs[pf::M_SR], c.ld, sys.nr, false);
    pad_store(lo.gml + p * B, c.gs[pf::M_GML], c.ld, sys.nl, false);
    pad_store(lo.gmr + p * B, c.gs[pf::M_GMR], c.ld, sys.nr, false);
    if (threadIdx.x == 0) {
      lead_status[p] = st;
      if (out.iters) {
        out.iters[2 * p] = itl;
        out.iters[2 * p + 1] = itr;
      }
    }
    __syncthreads();
  }
  pf::tc::small_release(tcx);
}



// Refinement residual r_j = b_j - A X (df64) of every point and every
// extended layer, written in FP32 into the forward-vector slab (the forward
// pass consumes r_j before it overwrites the slot with y_j).
//
// One CTA of kResThreads threads takes a run of kResLayers consecutive
// layers of one point.  The solution blocks X_{j-1}, X_j, X_{j+1} sit in a
// four-slot window of shared memory (X_j in slot j % 4); X_{j+2} is fetched
// into registers before layer j is computed and stored after it, so its
// global latency overlaps the arithmetic.  Thread (r, c0) computes row r of
// columns c0, c0 + 8, c0 + 16, c0 + 24: every ELL (or dense) entry of row r
// feeds four independent accumulators.
constexpr int kResThreads = 256;
constexpr int kResLayers = 8;
constexpr int kResCols = pf::wp::NW * pf::wp::NW / kResThreads;  // columns a thread
constexpr int kResColStep = kResThreads / pf::wp::NW;              // column stride
constexpr size_t kResSmem = 4 * (size_t)pf::wp::NW * pf::wp::NW * sizeof(dcx);

__device__ __forceinline__ void res_fetch(dcx (&v)[kResCols], const dcx* src) {
#pragma unroll
  for (int i = 0; i < kResCols; ++i) v[i] = src[threadIdx.x + i * kResThreads];
}
__device__ __forceinline__ void res_put(dcx* dst, const dcx (&v)[kResCols]) {
#pragma unroll
  for (int i = 0; i < kResCols; ++i) dst[threadIdx.x + i * kResThreads] = v[i];
}
// acc[i] += M(r, :) X(:, c0 + i*kResColStep) over the ELL row r of block blk
__device__ __forceinline__ void ell_acc4(const pf::Ell& e, size_t blk, int r, const dcx* X, int c0,
                                         dcx (&acc)[kResCols]) {
  for (int k = 0; k < e.K; ++k) {
    const size_t at = pf::ell_at(blk, e.K, e.rows, r, k);
    const int cc = e.col[at];
    if (cc < 0) break;
    const dcx v = e.val[at];
#pragma unroll
    for (int i = 0; i < kResCols; ++i) acc[i] = pf::cfma(v, X[cc + (c0 + i * kResColStep) * pf::wp::NW], acc[i]);
  }
}
// the same with a dense (ct: conjugate-transposed) global block
__device__ __forceinline__ void dense_acc4(const dcx* M, int ldm, int kdim, bool ct, int r, const dcx* X, int c0,
                                           dcx (&acc)[kResCols]) {
  for (int k = 0; k < kdim; ++k) {
    const dcx m = ct ? pf::cconj(M[k + (size_t)r * ldm]) : M[r + (size_t)k * ldm];
#pragma unroll
    for (int i = 0; i < kResCols; ++i) acc[i] = pf::cfma(m, X[k + (c0 + i * kResColStep) * pf::wp::NW], acc[i]);
  }
}

// Per-point energies in df64: zL = E + i eps, zD = E + i dev_factor eps.
__global__ void point_z_kernel(pf::Points pts, pf::Params P, dcx* z2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= pts.npts) return;
  const double E = pts.E[p];
  const double eps = E * P.eta + P.eta0;
  z2[2 * p] = pf::mk<pf::df64>(pf::df64(E), pf::df64(eps));
  z2[2 * p + 1] = pf::mk<pf::df64>(pf::df64(E), pf::df64(P.dev_factor * eps));
}

// Points whose last refinement sweep left a correction above PF_REFINE_TOL
// (order is irrelevant: every point is solved independently).
__global__ void refine_select_kernel(int npts, const float* corr, int* list, int* count) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npts || !(corr[p] > pf::PF_REFINE_TOL)) return;
  list[atomicAdd(count, 1)] = p;
}

template <bool kList>
__global__ void __launch_bounds__(kResThreads)
    residual_kernel(pf::MSys s, pf::Points pts, const dcx* z2, pf::wp::LeadOut lo, pf::wp::Slabs sl,
                    const int* list, const int* count) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  dcx* win = reinterpret_cast<dcx*>(smem_raw);
  constexpr int NW = pf::wp::NW;
  constexpr int B = NW * NW;
  const int L = s.L, n = s.n, nb = L + 2;
  const int r = threadIdx.x % NW, c0 = threadIdx.x / NW;
  const int runs = (nb + kResLayers - 1) / kResLayers;
  const bool sparse = s.ell_overflow != nullptr && *s.ell_overflow == 0;
  // kList: the points of an adaptive refinement sweep are list[0 .. *count)
  const int np = kList ? *count : pts.npts;
  for (int task = blockIdx.x; task < np * runs; task += gridDim.x) {
    const int p = kList ? list[task / runs] : task / runs;
    const int j0 = (task % runs) * kResLayers;
    const int j1 = j0 + kResLayers < nb ? j0 + kResLayers : nb;
    const int q = pts.qidx ? pts.qidx[p] : 0;
    const dcx* xb = sl.xv + (size_t)p * nb * B;
    fcx* yb = sl.yv + (size_t)p * nb * B;
    dcx nxt[kResCols];
    __syncthreads();  // the previous run is done with the window
    for (int jj = (j0 > 0 ? j0 - 1 : 0); jj <= j0 + 1 && jj < nb; ++jj) {
      res_fetch(nxt, xb + (size_t)jj * B);
      res_put(win + (jj & 3) * B, nxt);
    }
    __syncthreads();
    for (int j = j0; j < j1; ++j) {
      const bool more = j + 1 < j1 && j + 2 < nb;  // layer j+1 of this run needs X_{j+2}
      if (more) res_fetch(nxt, xb + (size_t)(j + 2) * B);
      const int dj = j == 0 ? s.nl : (j == L + 1 ? s.nr : n);
      const dcx* X0 = win + (j & 3) * B;
      const dcx* Xm = win + ((j + 3) & 3) * B;
      const dcx* Xp = win + ((j + 1) & 3) * B;
      fcx outv[kResCols];
#pragma unroll
      for (int i = 0; i < kResCols; ++i) outv[i] = pf::mk<float>(0.f, 0.f);
      if (r < dj) {
        const dcx z = z2[2 * p + (j == 0 ? 0 : 1)];
        dcx acc[kResCols];
#pragma unroll
        for (int i = 0; i < kResCols; ++i) {
          const int c = c0 + i * kResColStep;
          acc[i] = pf::csub(pf::wp::dz(), pf::cmul(z, X0[r + c * NW]));
          if (j == L + 1 && r == c) acc[i].x = acc[i].x + pf::df64(1.f, 0.f);
        }
        if (j == 0) {
          dense_acc4(lo.esl + (size_t)p * B, NW, s.nl, false, r, X0, c0, acc);
          if (sparse)
            ell_acc4(s.eHld, (size_t)q, r, Xp, c0, acc);
          else
            dense_acc4(s.Hld + (size_t)q * s.nl * n, s.nl, n, false, r, Xp, c0, acc);
        } else if (j <= L) {
          if (sparse) {
            ell_acc4(s.eHd, (size_t)q * L + (j - 1), r, X0, c0, acc);
            if (j == 1)
              ell_acc4(s.eHldH, (size_t)q, r, Xm, c0, acc);
            else
              ell_acc4(s.eHdvH, (size_t)q * (L - 1) + (j - 2), r, Xm, c0, acc);
            if (j == L)
              ell_acc4(s.eHrdH, (size_t)q, r, Xp, c0, acc);
            else
              ell_acc4(s.eHdv, (size_t)q * (L - 1) + (j - 1), r, Xp, c0, acc);
          } else {
            dense_acc4(s.Hd + ((size_t)q * L + (j - 1)) * n * n, n, n, false, r, X0, c0, acc);
            if (j == 1)
              dense_acc4(s.Hld + (size_t)q * s.nl * n, s.nl, s.nl, true, r, Xm, c0, acc);
            else
              dense_acc4(s.Hdv + ((size_t)q * (L - 1) + (j - 2)) * n * n, n, n, true, r, Xm, c0, acc);
            if (j == L)
              dense_acc4(s.Hrd + (size_t)q * s.nr * n, s.nr, s.nr, true, r, Xp, c0, acc);
            else
              dense_acc4(s.Hdv + ((size_t)q * (L - 1) + (j - 1)) * n * n, n, n, false, r, Xp, c0, acc);
          }
        } else {
          dense_acc4(s.HR + (size_t)q * s.nr * s.nr, s.nr, s.nr, false, r, X0, c0, acc);
          dense_acc4(lo.sr + (size_t)p * B, NW, s.nr, false, r, X0, c0, acc);
          if (sparse)
            ell_acc4(s.eHrd, (size_t)q, r, Xm, c0, acc);
          else
            dense_acc4(s.Hrd + (size_t)q * s.nr * n, s.nr, n, false, r, Xm, c0, acc);
        }
#pragma unroll
        for (int i = 0; i < kResCols; ++i)
          if (c0 + i * kResColStep < s.nr) outv[i] = pf::mk<float>(acc[i].x.hi, acc[i].y.hi);
      }
#pragma unroll
      for (int i = 0; i < kResCols; ++i) yb[(size_t)j * B + r + (c0 + i * kResColStep) * NW] = outv[i];
      if (more) res_put(win + ((j + 2) & 3) * B, nxt);
      __syncthreads();
    }
  }
}

constexpr int kSplitCols = pf::wp::NW / kWarpsPerCta;

// One refinement sweep of a point over the NC solution columns
// [cb, cb + NC): NC = 32 when a warp owns the point, kSplitCols when the
// warps of a CTA share it (the columns are independent right-hand sides).
//   forward:  y_j = g_j (r_j + V_{j-1}^H y_{j-1})   (r_j in yv[j] on entry)
//   backward: d_{L+1} = y_{L+1}; d_j = y_j + g_j V_j d_{j+1}; X += d
// md, mx: the largest |d_0| and |X_0| over rows < nl and these columns
// (warp-reduced).
template <int NC>
__device__ __forceinline__ void refine_sweep(const pf::MSys& sys, int q, int lane, int cb, fcx* X, fcx* Y,
                                             const fcx* lu, fcx* yv, dcx* xv, float& md, float& mx) {
  using namespace pf::wp;
  const int L = sys.L;
  const size_t B = (size_t)NW * NW;
  fcx a[NW];
#pragma unroll
  for (int i = 0; i < NC; ++i) Y[lane + (cb + i) * LDW] = yv[lane + (cb + i) * NW];
  __syncwarp();
  for (int j = 0; j <= L + 1; ++j) {
    if (j >= 1) {
      stage_rows(Y, vview(sys, q, j - 1), lane);
      __syncwarp();
      row_smem_h(Y, lane, a);                                    // row of V_{j-1}^H
      __syncwarp();
#pragma unroll
      for (int i = 0; i < NC; ++i) Y[lane + (cb + i) * LDW] = yv[(size_t)j * B + lane + (cb + i) * NW];   // r_j
      rgemm_cols<NC>(a, X, lane, cb, [&](int r, int c, fcx v) {  // u = r_j + V^H y_{j-1}
        Y[r + c * LDW] = pf::cadd(v, Y[r + c * LDW]);
      });
      __syncwarp();
    }
    row_block(lu + (size_t)j * B, lane, a);
    rgemm_cols<NC>(a, Y, lane, cb, [&](int r, int c, fcx v) {    // y_j = g_j u
      X[r + c * LDW] = v;
      yv[(size_t)j * B + r + c * NW] = v;
    });
    __syncwarp();
  }
#pragma unroll
  for (int i = 0; i < NC; ++i) {
    dcx& x = xv[(size_t)(L + 1) * B + lane + (cb + i) * NW];
    const fcx d = X[lane + (cb + i) * LDW];
    x.x = x.x + pf::df64(d.x, 0.f);
    x.y = x.y + pf::df64(d.y, 0.f);
  }
  for (int j = L; j >= 0; --j) {
    row_view(vview(sys, q, j), lane, a);
    rgemm_cols<NC>(a, X, lane, cb, [&](int r, int c, fcx v) { Y[r + c * LDW] = v; });  // t = V_j d_{j+1}
    __syncwarp();
    row_block(lu + (size_t)j * B, lane, a);
#pragma unroll
    for (int i = 0; i < NC; ++i) X[lane + (cb + i) * LDW] = yv[(size_t)j * B + lane + (cb + i) * NW];   // y_j
    rgemm_cols<NC>(a, Y, lane, cb, [&](int r, int c, fcx v) {    // d_j = y_j + g_j t
      X[r + c * LDW] = pf::cadd(v, X[r + c * LDW]);
    });
    // X += d, all loads of the row in flight together
#pragma unroll
    for (int i = 0; i < NC; ++i) {
      dcx& x = xv[(size_t)j * B + lane + (cb + i) * NW];
      const fcx d = X[lane + (cb + i) * LDW];
      x.x = x.x + pf::df64(d.x, 0.f);
      x.y = x.y + pf::df64(d.y, 0.f);
    }
    __syncwarp();
  }
  md = 0.f;
  mx = 0.f;
  if (lane < sys.nl) {
    for (int i = 0; i < NC; ++i) {
      const int c = cb + i;
      if (c >= sys.nr) break;
      const fcx d = X[lane + c * LDW];
      const dcx x = xv[lane + c * NW];
      md = fmaxf(md, fabsf(d.x) + fabsf(d.y));
      mx = fmaxf(mx, fabsf(x.x.hi) + fabsf(x.y.hi));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    md = fmaxf(md, __shfl_xor_sync(0xffffffffu, md, o));
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
}

__global__ void __launch_bounds__(kWarpsPerCta * 32, kLayerCtasPerSm)
    layer_kernel(pf::MSys sys, pf::Points pts, pf::Params P, int phase, pf::Outputs out, pf::wp::LeadOut lo,
                 pf::wp::Slabs sl, int* lead_status, int* queue, const int* list, const int* count) {
  using namespace pf::wp;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // two 32 x 32 FP32 buffers per warp
  fcx* X = reinterpret_cast<fcx*>(smem_raw) + (size_t)w * 2 * LDW * NW;
  fcx* Y = X + LDW * NW;
  const int L = sys.L, nr = sys.nr;
  const size_t B = (size_t)NW * NW;
  // list/count: the points of an adaptive refinement sweep (all points when null)
  const int np = list ? *count : pts.npts;
  // phase 3: a refinement sweep in which the CTA's warps share one point,
  // each taking kSplitCols of the solution's columns
  const bool split = (phase == 3);
  __shared__ int s_pi;
  __shared__ float2 s_red[kWarpsPerCta];
  for (;;) {
    int pi = 0;
    if (split) {
      __syncthreads();  // s_pi and s_red of the previous point are consumed
      if (threadIdx.x == 0) s_pi = atomicAdd(queue, 1);
      __syncthreads();
      pi = s_pi;
    } else {
      if (lane == 0) pi = atomicAdd(queue, 1);
      pi = __shfl_sync(0xffffffffu, pi, 0);
    }
    if (pi >= np) break;
    const int p = list ? list[pi] : pi;
    const int q = pts.qidx ? pts.qidx[p] : 0;
    const double E = pts.E[p];
    const double eps = E * P.eta + P.eta0;
    const fcx zf = pf::mk<float>((float)E, (float)(P.dev_factor * eps));
    int st = lead_status[p];
    const bool do_factor = (phase == 0), do_refine = (phase == 1 || split), do_caroli = (phase == 2);
    fcx* lu = sl.lu + (size_t)p * (L + 2) * B;
    fcx* yv = sl.yv + (size_t)p * (L + 2) * B;
    dcx* xv = sl.xv + (size_t)p * (L + 2) * B;
    fcx a[NW];
    const auto to_df = [](fcx v) { return pf::mk<pf::df64>(pf::df64(v.x, 0.f), pf::df64(v.y, 0.f)); };
    if (do_factor) {
      // ---- g_0 = gl (padded), kept in X and lu[0]
      const fcx* g0 = lo.g0 + p * B;
      for (int c = 0; c < NW; ++c) {
        const fcx v = g0[lane + c * NW];
        X[lane + c * LDW] = v;
        lu[lane + c * NW] = v;
      }
      __syncwarp();
      // ---- FP32 block LU, j = 1..L+1: A_j = z - H_j - V^H g_{j-1} V (- Sigma_R), g_j = A_j^-1
      for (int j = 1; j <= L + 1; ++j) {
        const int dj = edim(sys, j);
        row_smem(X, lane, a);                                    // row of g_{j-1}
        stage_rows(Y, vview(sys, q, j - 1), lane);                // V
        __syncwarp();
        rgemm(a, Y, lane, [&](int r, int c, fcx v) { X[r + c * LDW] = v; });  // T = g_{j-1} V
        __syncwarp();
        row_smem_h(Y, lane, a);                                  // row of V^H
        __syncwarp();
        const fcx* H = (j <= L) ? sys.fHd + ((size_t)q * L + (j - 1)) * sys.n * sys.n : sys.fHR + (size_t)q * nr * nr;
        const int ldh = (j <= L) ? sys.n : nr;
        const fcx* Sr = lo.fsr + p * B;
        // H_j (+ Sigma_R) into Y first: the loads of a whole row are in flight
        // together instead of one per epilogue column
#pragma unroll
        for (int c = 0; c < NW; ++c) {
          fcx h = fz();
          if (lane < dj && c < dj) {
            h = H[lane + (size_t)c * ldh];
            if (j == L + 1) h = pf::cadd(h, Sr[lane + c * NW]);
          }
          Y[lane + c * LDW] = h;
        }
        rgemm(a, X, lane, [&](int r, int c, fcx u) {             // A_j from V^H T
          fcx v;
          if (r < dj && c < dj) {
            v = pf::mk<float>(-u.x, -u.y);
            if (r == c) v = pf::cadd(v, zf);
            v = pf::csub(v, Y[r + c * LDW]);
          } else {
            v = pf::mk<float>(r == c ? 1.f : 0.f, 0.f);
          }
          Y[r + c * LDW] = v;
        });
        __syncwarp();
        st |= winverse(Y, X, lu + (size_t)j * B, lane);         // g_j -> X and lu[j]
      }
      // ---- back substitution: X_{L+1} = g_{L+1}; X_j = g_j V_j X_{j+1} (columns >= nr are zero)
      for (int c = 0; c < NW; ++c) {
        const fcx v = c < nr ? X[lane + c * LDW] : fz();
        X[lane + c * LDW] = v;
        xv[(size_t)(L + 1) * B + lane + c * NW] = to_df(v);
      }
      __syncwarp();
      for (int j = L; j >= 0; --j) {
        row_view(vview(sys, q, j), lane, a);
        rgemm(a, X, lane, [&](int r, int c, fcx v) { Y[r + c * LDW] = v; });  // W = V_j X_{j+1}
        __syncwarp();
        row_block(lu + (size_t)j * B, lane, a);
        rgemm(a, Y, lane, [&](int r, int c, fcx v) {             // X_j = g_j W
          if (c >= nr) v = fz();
          X[r + c * LDW] = v;
          xv[(size_t)j * B + r + c * NW] = to_df(v);
        });
        __syncwarp();
      }
    }  // do_factor
    // ---- one refinement sweep (the residual r_j was written into yv[j] by residual_kernel)
    if (do_refine) {
      float md, mx;
      if (split) {
        refine_sweep<kSplitCols>(sys, q, lane, w * kSplitCols, X, Y, lu, yv, xv, md, mx);
        if (lane == 0) s_red[w] = make_float2(md, mx);
        __syncthreads();
        if (threadIdx.x == 0) {
          for (int i = 1; i < kWarpsPerCta; ++i) {
            md = fmaxf(md, s_red[i].x);
            mx = fmaxf(mx, s_red[i].y);
          }
        }
      } else {
        refine_sweep<NW>(sys, q, lane, 0, X, Y, lu, yv, xv, md, mx);
      }
      const bool writer = split ? threadIdx.x == 0 : lane == 0;
      if (writer) sl.corr[p] = mx > 0.f ? md / mx : (md > 0.f ? INFINITY : 0.f);
    }
    if (do_factor) {
      if (lane == 0) lead_status[p] = st;
      continue;
    }
    if (do_refine) continue;
    // ---- Caroli in df64: lane c: P[:,c] = X0 GR[:,c]; Q[c,:] = X0[:,c]^H GL; tr += sum_r P[r,c] Q[c,r]
    double tr = 0.0;
    if (do_caroli) {
      const dcx* X0 = xv;
      const dcx* GR = lo.gmr + p * B;
      const dcx* GL = lo.gml + p * B;
      const int nl = sys.nl;
      if (lane < nr) {
        pf::df64 acc(0.f, 0.f);
        for (int r = 0; r < nl; ++r) {
          dcx pr = pf::wp::dz();
          for (int k = 0; k < nr; ++k) pr = pf::cfma(X0[r + k * NW], GR[k + lane * NW], pr);
          dcx qr = pf::wp::dz();
          for (int k = 0; k < nl; ++k) qr = pf::cfma(pf::cconj(X0[k + lane * NW]), GL[k + r * NW], qr);
          acc = acc + (pr.x * qr.x - pr.y * qr.y);
        }
        tr = pf::to_d(acc);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o);
    }
    if (lane == 0) {
      const bool zero = pts.zero_flag && pts.zero_flag[p];
      double v = tr;
      if (zero || v < 1.0e-60) v = 0.0;
      if (!(v == v)) st |= pf::PF_NAN;
      out.transl[p] = v;
      out.status[p] = st;
    }
  }
}

template <int S>
int mixed_grid(const MixedLayout& lay, int npts) {
  const int per_sm = pfn::fused_per_sm(S, lay.smem);
  if (per_sm < 1) return -1;
  DevInfo d = device_info();
  int g = d.sms * per_sm;
  return g < npts ? g : npts;
}

// Workspace plan of the mixed path (byte offsets into the caller's buffer).
struct MixedPlan {
  MixedLayout lay;
  bool warp_engine;     // cross-sections <= 32: leads kernel + warp-per-point layer kernel
  int grid_a, grid_b;   // CTA counts of the (leads / fused) kernel and the layer kernel
  int grid_r;           // resident CTAs of the residual kernel
  int grid_s;           // CTAs of the split refinement sweeps (a CTA per listed point)
  size_t per_cta_a;     // per-CTA scratch of kernel A
  size_t off_blocks, off_ell, off_scratch, off_lead, off_lstat, off_z, off_refine, off_slabs, total;
  size_t smem_b;
};

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

template <int S>
int leads_grid(const MixedLayout& lay, int npts) {
  auto k = leads_kernel<S>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.smem_leads) != cudaSuccess)
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, lay.smem_leads) != cudaSuccess) return -1;
  if (per_sm < 1) return -1;
  DevInfo d = device_info();
  int g = d.sms * per_sm;
  return g < npts ? g : npts;
}

bool make_plan(int n, int nl, int nr, int L, int nq, int npts, MixedPlan& P) {
  P.lay = make_mixed_layout(n, nl, nr, L, nq);
  const MixedLayout& lay = P.lay;
  const int S = (lay.base.m + 31) / 32;
  const int np = npts > 0 ? npts : 1;
  P.warp_engine = lay.base.m <= pf::wp::NW;
  const size_t Bn = (size_t)pf::wp::NW * pf::wp::NW;
  if (P.warp_engine) {
    P.grid_a = leads_grid<1>(lay, np);
    P.per_cta_a = al256((size_t)pf::NGM * lay.base.mat * 16 + 3 * lay.base.mat * 8);
    P.smem_b = (size_t)kWarpsPerCta * 2 * pf::wp::LDW * pf::wp::NW * 8;
    if (cudaFuncSetAttribute(layer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.smem_b) !=
        cudaSuccess)
      return false;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, layer_kernel, kWarpsPerCta * 32, P.smem_b) !=
            cudaSuccess ||
        per_sm < 1)
      return false;
    DevInfo d = device_info();
    const int warps = (np + 0);
    int gb = d.sms * per_sm;
    const int need_ctas = (warps + kWarpsPerCta - 1) / kWarpsPerCta;
    P.grid_b = gb < need_ctas ? gb : need_ctas;
    P.grid_s = gb < np ? gb : np;
    if (cudaFuncSetAttribute(residual_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kResSmem) != cudaSuccess ||
        cudaFuncSetAttribute(residual_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kResSmem) !=
            cudaSuccess)
      return false;
    int per_sm_r = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_r, residual_kernel<false>, kResThreads, kResSmem) !=
            cudaSuccess ||
        per_sm_r < 1)
      return false;
    P.grid_r = d.sms * per_sm_r;
  } else {
    P.grid_a = mixed_grid<2>(lay, np);  // 32 < m <= 64
    P.per_cta_a = lay.per_cta;
    P.grid_b = 0;
    P.grid_r = 0;
    P.grid_s = 0;
    P.smem_b = 0;
  }
  if (P.grid_a <= 0) return false;
  size_t o = 256;  // work queues
  P.off_blocks = o;
  o += lay.blocks_d + lay.blocks_f;
  P.off_ell = o;
  o += lay.ell_bytes;
  P.off_scratch = o;
  o += (size_t)P.grid_a * P.per_cta_a;
  P.off_lead = o;
  if (P.warp_engine) o += al256((size_t)np * Bn * (8 + 8 + 16 * 4));
  P.off_lstat = o;
  if (P.warp_engine) o += al256((size_t)np * sizeof(int));
  P.off_z = o;
  if (P.warp_engine) o += al256((size_t)np * 2 * 16);
  P.off_refine = o;  // per-point relative corrections and the compacted point list
  if (P.warp_engine) o += al256((size_t)np * 2 * sizeof(int));
  P.off_slabs = o;
  if (P.warp_engine) o += al256((size_t)np * (L + 2) * Bn * (8 + 8 + 16));
  P.total = o;
  return true;
}

size_t mixed_workspace_bytes(int n, int nl, int nr, int L, int nq, int npts) {
  MixedPlan P;
  if (!make_plan(n, nl, nr, L, nq, npts, P)) return 0;
  return P.total;
}

}  // namespace

extern "C" {
size_t pf_transport_tdb_mixed_workspace_size(int n, int nl, int nr, int L, int nq, int npts) {
  if (check_dims(n, nl, nr, L, nq, npts) != PF_SUCCESS) return 0;
  return mixed_workspace_bytes(n, nl, nr, L, nq, npts);
}
}  // extern "C"


namespace {
// One pass of the mixed pipeline over npts points with the workspace `work`
// laid out by `plan` (made for at least npts points), on stream st.
// Optional stage timing of the mixed pipeline (pf_mixed_stage_timing):
// events recorded on the call's stream before the block conversions, around
// the lead decimations and after the last sweep.  One set per process; the
// calls being timed must not overlap and must not be captured into a graph.
struct StageTimer {
  bool on = false;
  bool ready = false;
  bool recorded = false;
  cudaEvent_t ev[4];
  void mark(int i, cudaStream_t st) {
    if (!on) return;
    if (!ready) {
      for (auto& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) return;
      ready = true;
    }
    cudaEventRecord(ev[i], st);
    if (i == 3) recorded = true;
  }
};
StageTimer g_timer;

int mixed_launch(const MixedPlan& plan, int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                 const double* HR, const double* HRv, const double* Hd, const double* Hdv, const double* Hld,
                 const double* Hrd, int npts, const double* E, const int* qidx, const int* zero_flag, double eta,
                 double eta0, double dev_factor, double convergence, int max_iter, int refine_iters, int lead_mode,
                 double* transl, int* status, int* iters, void* work, cudaStream_t st) {
  const MixedLayout& lay = plan.lay;
  const int S = (lay.base.m + 31) / 32;
  char* w = reinterpret_cast<char*>(work);
  int* queue = reinterpret_cast<int*>(w);
  int* queue_b = queue + 1;
  char* p = w + plan.off_blocks;
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
  // ELL copies of the device-side blocks (residual of the refinement)
  p = w + plan.off_ell;
  int* ell_over = reinterpret_cast<int*>(p);
  p += 256;
  int* ecol[7];
  dcx* eval[7];
  for (int i = 0; i < 7; ++i) {
    ecol[i] = reinterpret_cast<int*>(p);
    p += (lay.ell_rows[i] * pf::PF_ELL_K * 4 + 255) & ~(size_t)255;
    eval[i] = reinterpret_cast<dcx*>(p);
    p += (lay.ell_rows[i] * pf::PF_ELL_K * 16 + 255) & ~(size_t)255;
  }
  int* mirror = reinterpret_cast<int*>(p);
  char* scratch = w + plan.off_scratch;
  g_timer.mark(0, st);
  for (int i = 0; i < 8; ++i) {
    if (lay.cnt[i] == 0) continue;
    const int blocks = (int)((lay.cnt[i] + 255) / 256 < 4096 ? (lay.cnt[i] + 255) / 256 : 4096);
    convert_blocks_kernel<<<blocks, 256, 0, st>>>(reinterpret_cast<const cx<double>*>(src[i]), dd[i],
                                                   i >= 2 ? ff[i] : nullptr, lay.cnt[i]);
  }
  PF_CUDA(cudaGetLastError());
  PF_CUDA(cudaMemsetAsync(ell_over, 0, sizeof(int), st));
  {
    struct F {
      const dcx* m;
      int rows, cols, count, ct;
    } fam[7] = {{dd[4], n, n, nq * L, 0},           {dd[5], n, n, nq * (L - 1), 0}, {dd[5], n, n, nq * (L - 1), 1},
                {dd[6], nl, n, nq, 0},              {dd[6], nl, n, nq, 1},          {dd[7], nr, n, nq, 0},
                {dd[7], nr, n, nq, 1}};
    for (int i = 0; i < 7; ++i) {
      if (lay.ell_rows[i] == 0) continue;
      const int blocks = (int)((lay.ell_rows[i] + 127) / 128 < 4096 ? (lay.ell_rows[i] + 127) / 128 : 4096);
      build_ell_kernel<<<blocks, 128, 0, st>>>(fam[i].m, fam[i].rows, fam[i].cols, fam[i].count, fam[i].ct,
                                                pf::PF_ELL_K, ecol[i], eval[i], ell_over);
    }
    PF_CUDA(cudaGetLastError());
  }
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
  sys.dHL = reinterpret_cast<const cx<double>*>(HL);
  sys.dHLv = reinterpret_cast<const cx<double>*>(HLv);
  sys.dHR = reinterpret_cast<const cx<double>*>(HR);
  sys.dHRv = reinterpret_cast<const cx<double>*>(HRv);
  sys.lead_mode = lead_mode;
  sys.fHR = ff[2];
  sys.fHd = ff[4];
  sys.fHdv = ff[5];
  sys.fHld = ff[6];
  sys.fHrd = ff[7];
  {
    const int rows[7] = {n, n, n, nl, n, nr, n};
    pf::Ell* es[7] = {&sys.eHd, &sys.eHdv, &sys.eHdvH, &sys.eHld, &sys.eHldH, &sys.eHrd, &sys.eHrdH};
    for (int i = 0; i < 7; ++i) {
      es[i]->col = ecol[i];
      es[i]->val = eval[i];
      es[i]->K = pf::PF_ELL_K;
      es[i]->rows = rows[i];
    }
    sys.ell_overflow = ell_over;
  }
  pf::Points pts{npts, E, qidx, zero_flag};
  pf::Params P{nullptr, eta, eta0, dev_factor, convergence, max_iter, 0};
  if (nl == nr) {
    lead_mirror_kernel<<<nq, 256, 0, st>>>(HL, HLv, HR, HRv, 2 * nl * nl, nq, mirror);
    P.lead_mirror = mirror;
  }
  pf::Outputs out{transl, nullptr, status, iters};
  PF_CUDA(cudaMemsetAsync(queue, 0, 2 * sizeof(int), st));
  if (plan.warp_engine) {
    const size_t Bn = (size_t)pf::wp::NW * pf::wp::NW;
    const size_t np = (size_t)npts;
    char* lp = w + plan.off_lead;
    pf::wp::LeadOut lo;
    lo.g0 = reinterpret_cast<fcx*>(lp);
    lo.fsr = lo.g0 + np * Bn;
    lo.esl = reinterpret_cast<dcx*>(lo.fsr + np * Bn);
    lo.sr = lo.esl + np * Bn;
    lo.gml = lo.sr + np * Bn;
    lo.gmr = lo.gml + np * Bn;
    int* lstat = reinterpret_cast<int*>(w + plan.off_lstat);
    pf::wp::Slabs sl;
    sl.lu = reinterpret_cast<fcx*>(w + plan.off_slabs);
    sl.yv = sl.lu + np * (L + 2) * Bn;
    sl.xv = reinterpret_cast<dcx*>(sl.yv + np * (L + 2) * Bn);
    sl.corr = reinterpret_cast<float*>(w + plan.off_refine);
    int* rlist = reinterpret_cast<int*>(sl.corr + np);
    int* rcount = queue + 2;
    if (lead_mode == pf::PF_LEAD_FP64) {
      // tensor-core products in the FP64 decimations: one CTA per SM
      const DevInfo di = device_info();
      size_t smem_tc = lay.smem_leads + 1024 + (size_t)pf::tc::kSmallSmem;
      const size_t gs_bytes = (size_t)kLeadsTcShared * lay.base.mat * sizeof(dcx);
      const int gs_smem = smem_tc + gs_bytes <= di.smem_optin ? 1 : 0;
      if (gs_smem) smem_tc += gs_bytes;
      PF_CUDA(cudaFuncSetAttribute(leads_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_tc));
      const int grid_tc = plan.grid_a < di.sms ? plan.grid_a : di.sms;
      g_timer.mark(1, st);
      leads_tc_kernel<<<grid_tc, kThreads, smem_tc, st>>>(sys, pts, P, out, lay, plan.per_cta_a, scratch, lo, lstat,
                                                          queue, gs_smem);
    } else {
      g_timer.mark(1, st);
      leads_kernel<1><<<plan.grid_a, kThreads, lay.smem_leads, st>>>(sys, pts, P, out, lay, plan.per_cta_a, scratch,
                                                                      lo, lstat, queue);
    }
    g_timer.mark(2, st);
    PF_CUDA(cudaGetLastError());
    // factorisation + back substitution, then each refinement sweep as a
    // parallel residual kernel followed by the warp-per-point correction,
    // then the Caroli trace
    layer_kernel<<<plan.grid_b, kWarpsPerCta * 32, plan.smem_b, st>>>(sys, pts, P, 0, out, lo, sl, lstat, queue_b,
                                                                       nullptr, nullptr);
    PF_CUDA(cudaGetLastError());
    const long rtasks = (long)npts * ((L + 2 + kResLayers - 1) / kResLayers);
    const int rblocks = (int)(rtasks < (long)plan.grid_r ? rtasks : (long)plan.grid_r);
    dcx* z2 = reinterpret_cast<dcx*>(w + plan.off_z);
    if (refine_iters > 0) point_z_kernel<<<(npts + 127) / 128, 128, 0, st>>>(pts, P, z2);
    for (int it = 0; it < refine_iters; ++it) {
      // the first sweep covers every point, later ones the points whose
      // previous correction was above PF_REFINE_TOL (grids sized for all
      // points; the kernels read the count on the device)
      const int* lst = nullptr;
      const int* cnt = nullptr;
      if (it > 0) {
        PF_CUDA(cudaMemsetAsync(rcount, 0, sizeof(int), st));
        refine_select_kernel<<<(npts + 255) / 256, 256, 0, st>>>(npts, sl.corr, rlist, rcount);
        lst = rlist;
        cnt = rcount;
      }
      if (it > 0)
        residual_kernel<true><<<rblocks, kResThreads, kResSmem, st>>>(sys, pts, z2, lo, sl, lst, cnt);
      else
        residual_kernel<false><<<rblocks, kResThreads, kResSmem, st>>>(sys, pts, z2, lo, sl, nullptr, nullptr);
      PF_CUDA(cudaMemsetAsync(queue_b, 0, sizeof(int), st));
      // later sweeps cover few points: a CTA per point, its warps splitting
      // the columns, shortens each point's sequential sweep
      layer_kernel<<<it > 0 ? plan.grid_s : plan.grid_b, kWarpsPerCta * 32, plan.smem_b, st>>>(
          sys, pts, P, it > 0 ? 3 : 1, out, lo, sl, lstat, queue_b, lst, cnt);
      PF_CUDA(cudaGetLastError());
    }
    PF_CUDA(cudaMemsetAsync(queue_b, 0, sizeof(int), st));
    layer_kernel<<<plan.grid_b, kWarpsPerCta * 32, plan.smem_b, st>>>(sys, pts, P, 2, out, lo, sl, lstat, queue_b,
                                                                       nullptr, nullptr);
    g_timer.mark(3, st);
  } else {
    PF_CUDA(pfn::fused_launch(S, plan.grid_a, lay.smem, st, sys, pts, P, refine_iters, out, lay, scratch, queue));
  }
  PF_CUDA(cudaGetLastError());
  return PF_SUCCESS;
}

int mixed_ex(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv, const double* HR,
             const double* HRv, const double* Hd, const double* Hdv, const double* Hld, const double* Hrd, int npts,
             const double* E, const int* qidx, const int* zero_flag, double eta, double eta0, double dev_factor,
             double convergence, int max_iter, int refine_iters, int lead_arith, double* transl, int* status,
             int* iters, void* work, size_t work_bytes, void* stream) {
  int rc = check_dims(n, nl, nr, L, nq, npts);
  if (rc != PF_SUCCESS) return rc;
  if (lead_arith == PF_ARITH_AUTO) {
    // FP64 decimations where their block products run on the tensor cores
    const int mx = nl > nr ? nl : nr;
    lead_arith = mx <= pf::tc::kSmallN && n <= pf::wp::NW ? PF_ARITH_FP64 : PF_ARITH_DF64;
  }
  if (lead_arith != PF_ARITH_FP64 && lead_arith != PF_ARITH_DF64 && lead_arith != PF_ARITH_SPLIT)
    return set_err(PF_ERR_ARG, "pf: lead_arith must be PF_ARITH_AUTO, PF_ARITH_FP64, PF_ARITH_DF64 or PF_ARITH_SPLIT");
  if (!E || !transl || !status) return set_err(PF_ERR_ARG, "pf: null energy/output pointer");
  if (!HL || !HLv || !HR || !HRv || !Hd || !Hld || !Hrd || (L > 1 && !Hdv))
    return set_err(PF_ERR_ARG, "pf: null block pointer");
  if (max_iter <= 0 || refine_iters < 0 || refine_iters > 16)
    return set_err(PF_ERR_ARG, "pf: max_iter must be positive and refine_iters in [0, 16]");
  if (npts == 0) return PF_SUCCESS;
  const int lead_mode = lead_arith == PF_ARITH_FP64 ? pf::PF_LEAD_FP64
                                                    : (lead_arith == PF_ARITH_DF64 ? pf::PF_LEAD_DF64 : pf::PF_LEAD_SPLIT);
  MixedPlan plan;
  if (!make_plan(n, nl, nr, L, nq, npts, plan)) return set_err(PF_ERR_SIZE, "pf: kernel does not fit on the device");
  DevInfo d = device_info();
  if (plan.lay.smem > d.smem_optin) return set_err(PF_ERR_SIZE, "pf: working set exceeds shared memory");
  if (!work || work_bytes < plan.total) return set_err(PF_ERR_ARG, "pf: workspace too small");
  return mixed_launch(plan, n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd, npts, E, qidx, zero_flag, eta,
                      eta0, dev_factor, convergence, max_iter, refine_iters, lead_mode, transl, status, iters, work,
                      (cudaStream_t)stream);
}
}  // namespace

extern "C" {
int pf_mixed_stage_timing(int on) {
  g_timer.on = on != 0;
  g_timer.recorded = false;
  return PF_SUCCESS;
}

int pf_mixed_stage_times(float* ms, int n) {
  if (!ms || n < 3) return set_err(PF_ERR_ARG, "pf_mixed_stage_times: need room for three durations");
  if (!g_timer.ready || !g_timer.recorded)
    return set_err(PF_ERR_ARG, "pf_mixed_stage_times: no timed call of the 32-wide pipeline");
  PF_CUDA(cudaEventSynchronize(g_timer.ev[3]));
  for (int i = 0; i < 3; ++i) PF_CUDA(cudaEventElapsedTime(&ms[i], g_timer.ev[i], g_timer.ev[i + 1]));
  return 3;
}

int pf_transport_tdb_mixed_ex_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                                  const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                                  const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                                  const int* zero_flag, double eta, double eta0, double dev_factor,
                                  double convergence, int max_iter, int refine_iters, int lead_arith,
                                  double* transl, int* status, int* iters, void* work, size_t work_bytes,
                                  void* stream) {
  return mixed_ex(n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd, npts, E, qidx, zero_flag, eta, eta0,
                  dev_factor, convergence, max_iter, refine_iters, lead_arith, transl, status, iters, work,
                  work_bytes, stream);
}

int pf_transport_tdb_mixed_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                               const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                               const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                               const int* zero_flag, double eta, double eta0, double dev_factor,
                               double convergence, int max_iter, int refine_iters, double* transl, int* status,
                               int* iters, void* work, size_t work_bytes, void* stream) {
  return mixed_ex(n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd, npts, E, qidx, zero_flag, eta, eta0,
                  dev_factor, convergence, max_iter, refine_iters, PF_ARITH_AUTO, transl, status, iters, work,
                  work_bytes, stream);
}
}  // extern "C"
