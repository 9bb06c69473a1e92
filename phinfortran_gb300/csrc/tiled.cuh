// Layer-synchronous batched kernels for block sizes beyond the resident
// (shared-memory) kernels: a batch of points advances through the same
// step together, every step one launch over the whole batch.
//
//   bgemm        : C_b = alpha op(A_b) op(B_b) + beta C_b [+ z_b I - H]
//                  column-major complex, 64x64 output tile per CTA, 256
//                  threads with a 4x4 complex register tile each, K staged
//                  through shared memory in steps of 8.  A stride of 0 shares
//                  an operand across the batch (the Gamma-point blocks), an
//                  optional per-point mask skips retired points.
//   inv_small    : in-place Gauss-Jordan inverse with partial pivoting of a
//                  matrix that fits in shared memory (one CTA per point).
//   gje_panel / gje_swap / gje_restore / gje_unpermute : the blocked
//                  Gauss-Jordan inverse (panel of nb columns factored in
//                  shared memory, the rest updated by bgemm).
#pragma once
#include <cuda_runtime.h>

#include "cmat.cuh"

namespace pf {
namespace tiled {

template <typename T>
struct GemmArgs {
  int m, n, k;
  const cx<T>* A;
  int lda;
  long long sA;
  const cx<T>* B;
  int ldb;
  long long sB;
  cx<T>* C;
  int ldc;
  long long sC;
  cx<T> alpha, beta;
  const int* active;  // per batch element (nullable): 0 -> skip
  // optional shift epilogue: C += z_b I - H_b
  const cx<T>* zdiag;  // per batch element (nullable)
  const cx<T>* H;      // nullable
  int ldh;
  long long sH;
};

constexpr int BM = 64, BN = 64, BK = 8, GT = 256;

// C = alpha * opA(A) * opB(B) + beta * C  (+ shift); CA / CB: conjugate-transpose
template <typename T, bool CA, bool CB>
__global__ void __launch_bounds__(GT) bgemm(GemmArgs<T> g) {
  const int b = blockIdx.z;
  if (g.active && !g.active[b]) return;
  // raw storage: cx<df64> has a constructor, shared arrays must not
  __shared__ __align__(16) unsigned char sa_raw[BK * (BM + 1) * sizeof(cx<T>)];
  __shared__ __align__(16) unsigned char sb_raw[BK * (BN + 1) * sizeof(cx<T>)];
  auto sa = reinterpret_cast<cx<T>(*)[BM + 1]>(sa_raw);
  auto sb = reinterpret_cast<cx<T>(*)[BN + 1]>(sb_raw);
  const cx<T>* A = g.A + (size_t)b * g.sA;
  const cx<T>* B = g.B + (size_t)b * g.sB;
  cx<T>* C = g.C + (size_t)b * g.sC;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int tid = threadIdx.x;
  const int tr = tid & 15, tc = tid >> 4;  // rows tr + 16 i, cols tc + 16 j
  cx<T> acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = mk<T>(T(0), T(0));
  for (int k0 = 0; k0 < g.k; k0 += BK) {
    // A tile: BM x BK (512 elements, 2 per thread)
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const int e = tid + t * GT;
      int r, kk;
      if (!CA) {
        r = e % BM;
        kk = e / BM;
      } else {
        kk = e % BK;
        r = e / BK;
      }
      const int gr = m0 + r, gk = k0 + kk;
      cx<T> v = mk<T>(T(0), T(0));
      if (gr < g.m && gk < g.k) v = CA ? cconj(A[gk + (size_t)gr * g.lda]) : A[gr + (size_t)gk * g.lda];
      sa[kk][r] = v;
    }
    // B tile: BK x BN
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const int e = tid + t * GT;
      int kk, c;
      if (!CB) {
        kk = e % BK;
        c = e / BK;
      } else {
        c = e % BN;
        kk = e / BN;
      }
      const int gk = k0 + kk, gc = n0 + c;
      cx<T> v = mk<T>(T(0), T(0));
      if (gk < g.k && gc < g.n) v = CB ? cconj(B[gc + (size_t)gk * g.ldb]) : B[gk + (size_t)gc * g.ldb];
      sb[kk][c] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      cx<T> a[4], bb[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sa[kk][tr + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bb[j] = sb[kk][tc + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = cfma(a[i], bb[j], acc[i][j]);
    }
    __syncthreads();
  }
  const bool use_beta = !(g.beta.x == T(0) && g.beta.y == T(0));
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = m0 + tr + 16 * i;
    if (r >= g.m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = n0 + tc + 16 * j;
      if (c >= g.n) continue;
      cx<T> v = cmul(g.alpha, acc[i][j]);
      if (use_beta) v = cfma(g.beta, C[r + (size_t)c * g.ldc], v);
      if (g.H) v = csub(v, g.H[(size_t)b * g.sH + r + (size_t)c * g.ldh]);
      if (g.zdiag && r == c) v = cadd(v, g.zdiag[b]);
      C[r + (size_t)c * g.ldc] = v;
    }
  }
}

// In-place inverse of an n x n matrix per batch element, staged through
// shared memory (ld = n | 1); status bits OR-ed into status[b].
template <typename T>
__global__ void __launch_bounds__(256) inv_small(cx<T>* A, int lda, long long sA, int n, const int* active,
                                                 int* status) {
  const int b = blockIdx.x;
  if (active && !active[b]) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ld = n | 1;
  cx<T>* M = reinterpret_cast<cx<T>*>(smem_raw);
  InvWork<T> w;
  w.rowk = M + (size_t)ld * n;
  w.colk = w.rowk + n;
  w.perm = reinterpret_cast<int*>(w.colk + n);
  w.flag = w.perm + n;
  cx<T>* G = A + (size_t)b * sA;
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
    const int r = i % n, c = i / n;
    M[r + c * ld] = G[r + (size_t)c * lda];
  }
  __syncthreads();
  const int st = inverse(M, ld, n, w);
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
    const int r = i % n, c = i / n;
    G[r + (size_t)c * lda] = M[r + c * ld];
  }
  if (threadIdx.x == 0 && st && status) atomicOr(&status[b], st);
}

// Blocked Gauss-Jordan, panel step: the n x nb panel A[:, k:k+nb] is
// factored in shared memory (pivot search over rows k+c.., row swaps inside
// the panel, scaling, elimination of every other row); the row swaps are
// recorded in piv[b][k+c] and applied to the other columns by gje_swap.
// The factored panel is written back to A and to P (restore copy); the
// pivot-row block M11 = A[k:k+nb, k:k+nb] goes to M11.
template <typename T>
__global__ void __launch_bounds__(256) gje_panel(cx<T>* A, int lda, long long sA, int n, int k, int nb, int* piv,
                                                 cx<T>* P, cx<T>* M11, const int* active, int* status) {
  const int b = blockIdx.x;
  if (active && !active[b]) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* S = reinterpret_cast<cx<T>*>(smem_raw);  // n x nb, ld = n
  cx<T>* colc = S + (size_t)n * nb;               // pivot column of the current step
  __shared__ __align__(16) unsigned char prow_raw[64 * sizeof(cx<T>)];
  cx<T>* prow = reinterpret_cast<cx<T>*>(prow_raw);
  __shared__ double rbest[8];
  __shared__ int ridx[8];
  __shared__ int s_p;
  cx<T>* G = A + (size_t)b * sA;
  int* pv = piv + (size_t)b * n;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < n * nb; i += nt) {
    const int r = i % n, c = i / n;
    S[r + (size_t)c * n] = G[r + (size_t)(k + c) * lda];
  }
  __syncthreads();
  int st = 0;
  for (int c = 0; c < nb; ++c) {
    const int col = k + c;
    // pivot search (first maximum of |re|+|im|; NaN wins)
    double best = -1.0;
    int bi = col;
    for (int i = col + tid; i < n; i += nt) {
      const double v = cabs1(S[i + (size_t)c * n]);
      const double vv = (v != v) ? 3.0e300 : v;
      if (vv > best) {
        best = vv;
        bi = i;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (lane == 0) {
      rbest[warp] = best;
      ridx[warp] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      double bb = rbest[0];
      int ii = ridx[0];
      for (int w = 1; w < (nt >> 5); ++w)
        if (rbest[w] > bb || (rbest[w] == bb && ridx[w] < ii)) {
          bb = rbest[w];
          ii = ridx[w];
        }
      s_p = ii;
      pv[col] = ii;
    }
    __syncthreads();
    const int p = s_p;
    if (p != col) {
      for (int j = tid; j < nb; j += nt) {
        const cx<T> t = S[col + (size_t)j * n];
        S[col + (size_t)j * n] = S[p + (size_t)j * n];
        S[p + (size_t)j * n] = t;
      }
    }
    __syncthreads();
    const cx<T> pivv = S[col + (size_t)c * n];
    if (pivv.x == T(0) && pivv.y == T(0)) st |= PF_SINGULAR;
    if (!(isfinite(pivv.x) && isfinite(pivv.y))) st |= PF_NAN;
    const cx<T> ip = crecip(pivv);
    for (int j = tid; j < nb; j += nt) prow[j] = (j == c) ? ip : cmul(S[col + (size_t)j * n], ip);
    for (int r = tid; r < n; r += nt) colc[r] = S[r + (size_t)c * n];
    __syncthreads();
    for (int i = tid; i < n * nb; i += nt) {
      const int r = i % n, j = i / n;
      if (r == col) {
        S[r + (size_t)j * n] = prow[j];
      } else {
        const cx<T> f = colc[r];
        if (j == c) {
          const cx<T> t = cmul(f, ip);
          S[r + (size_t)j * n] = mk<T>(-t.x, -t.y);
        } else {
          // v - f prow_j as two fused multiply-adds a component (four FP64
          // operations an element instead of six)
          const cx<T> pj = prow[j];
          cx<T> v = S[r + (size_t)j * n];
          v.x = fma(-f.x, pj.x, fma(f.y, pj.y, v.x));
          v.y = fma(-f.x, pj.y, fma(-f.y, pj.x, v.y));
          S[r + (size_t)j * n] = v;
        }
      }
    }
    __syncthreads();
  }
  cx<T>* Pb = P + (size_t)b * n * nb;
  cx<T>* Mb = M11 + (size_t)b * nb * nb;
  for (int i = tid; i < n * nb; i += nt) {
    const int r = i % n, c = i / n;
    const cx<T> v = S[r + (size_t)c * n];
    G[r + (size_t)(k + c) * lda] = v;
    Pb[i] = v;
    if (r >= k && r < k + nb) Mb[(r - k) + (size_t)c * nb] = v;
  }
  if (tid == 0 && st && status) atomicOr(&status[b], st);
}

// Row swaps of panel step k applied to the columns outside the panel; W
// receives the (swapped) pivot rows A[k:k+nb, :] (nb x n, ld nb).
template <typename T>
__global__ void gje_swap(cx<T>* A, int lda, long long sA, int n, int k, int nb, const int* piv, cx<T>* W,
                         const int* active) {
  const int b = blockIdx.y;
  if (active && !active[b]) return;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  cx<T>* G = A + (size_t)b * sA;
  const int* pv = piv + (size_t)b * n;
  const bool in_panel = (j >= k && j < k + nb);
  if (!in_panel) {
    for (int c = 0; c < nb; ++c) {
      const int r = k + c, p = pv[r];
      if (p != r) {
        const cx<T> t = G[r + (size_t)j * lda];
        G[r + (size_t)j * lda] = G[p + (size_t)j * lda];
        G[p + (size_t)j * lda] = t;
      }
    }
  }
  cx<T>* Wb = W + (size_t)b * nb * n;
  for (int c = 0; c < nb; ++c) Wb[c + (size_t)j * nb] = G[(k + c) + (size_t)j * lda];
}

// Panel columns back from the restore copy (the block updates touched them).
template <typename T>
__global__ void gje_restore(cx<T>* A, int lda, long long sA, int n, int k, int nb, const cx<T>* P,
                            const int* active) {
  const int b = blockIdx.y;
  if (active && !active[b]) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * nb) return;
  const int r = i % n, c = i / n;
  A[(size_t)b * sA + r + (size_t)(k + c) * lda] = P[(size_t)b * n * nb + i];
}

// Undo the row interchanges as column interchanges, last first.
template <typename T>
__global__ void gje_unpermute(cx<T>* A, int lda, long long sA, int n, const int* piv, const int* active) {
  const int b = blockIdx.x;
  if (active && !active[b]) return;
  cx<T>* G = A + (size_t)b * sA;
  const int* pv = piv + (size_t)b * n;
  for (int c = n - 1; c >= 0; --c) {
    const int p = pv[c];
    if (p != c) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const cx<T> t = G[i + (size_t)c * lda];
        G[i + (size_t)c * lda] = G[i + (size_t)p * lda];
        G[i + (size_t)p * lda] = t;
      }
    }
    __syncthreads();
  }
}

}  // namespace tiled
}  // namespace pf
