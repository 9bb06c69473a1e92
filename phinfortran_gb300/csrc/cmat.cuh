// CTA-level complex dense-matrix toolkit for the NEGF kernels (sm_103a).
//
// One CTA owns one (omega, q) point at a time.  Matrices are column-major
// (Fortran order, element (r,c) at p[r + c*ld]) and interleaved complex,
// exactly the layout of the reference's complex(kind=8) arrays.  Working
// matrices live in shared memory with an odd leading dimension, which makes
// both row-strided and column-contiguous warp accesses bank-conflict free.
//
// Primitives (all called by every thread of the CTA, all end with a barrier):
//   row_gemm  : C[r,:] = sum_k opA(r,k) opB(k,:)   one warp per output row;
//               the warp holds row r of opA in registers first, so C may
//               alias A (in-place right-multiplication, opA = N only).
//   inverse   : in-place Gauss-Jordan with partial (row) pivoting, the
//               pivot chosen by |re|+|im| like LAPACK's izamax.
// Non-conjugated operands must be in shared memory (their warp access is
// strided); conjugate-transposed operands may be in global memory (their
// warp access is contiguous).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "df64.cuh"

namespace pf {

template <typename R>
struct alignas(2 * sizeof(R)) cx {
  R x, y;
};

template <typename R>
__device__ __forceinline__ cx<R> mk(R a, R b) {
  cx<R> z;
  z.x = a;
  z.y = b;
  return z;
}
template <typename R>
__device__ __forceinline__ cx<R> czero() {
  return mk<R>(R(0), R(0));
}
template <typename R>
__device__ __forceinline__ cx<R> cadd(cx<R> a, cx<R> b) {
  return mk<R>(a.x + b.x, a.y + b.y);
}
template <typename R>
__device__ __forceinline__ cx<R> csub(cx<R> a, cx<R> b) {
  return mk<R>(a.x - b.x, a.y - b.y);
}
template <typename R>
__device__ __forceinline__ cx<R> cconj(cx<R> a) {
  return mk<R>(a.x, -a.y);
}
template <typename R>
__device__ __forceinline__ cx<R> cmul(cx<R> a, cx<R> b) {
  return mk<R>(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a*b + c
template <typename R>
__device__ __forceinline__ cx<R> cfma(cx<R> a, cx<R> b, cx<R> c) {
  return mk<R>(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
// Dot-product accumulator of row_gemm.  For float and double it is a plain
// fused multiply-add.  For df64 it follows the compensated dot product of
// Ogita, Rump and Oishi ("Accurate sum and dot product", SIAM J. Sci.
// Comput. 26, 2005, Algorithm Dot2): the high parts of the products are
// summed with TwoSum into one float and the rounding errors, with the df64
// cross terms, into a second float.  Unlike Dot2 the pair is renormalised
// after every complex term (two real terms per part), which keeps the error
// float small and the accuracy that of a normalised df64 sum -- 13.5 FP32
// operations a real term instead of the 15 of a df64 fma.
template <typename R>
struct Acc {
  cx<R> v;
  __device__ __forceinline__ void zero() { v = czero<R>(); }
  __device__ __forceinline__ void mac(cx<R> a, cx<R> b) { v = cfma(a, b, v); }
  __device__ __forceinline__ cx<R> get() const { return v; }
};
struct Dot2 {
  float h, l;
  __device__ __forceinline__ void add(float xh, float xl, df64 y) {  // += x*y
    const float p = __fmul_rn(xh, y.hi);
    float e = __fmaf_rn(xh, y.hi, -p);
    e = __fmaf_rn(xh, y.lo, e);
    e = __fmaf_rn(xl, y.hi, e);
    const float s = __fadd_rn(h, p);
    const float v = __fsub_rn(s, h);
    const float t = __fadd_rn(__fsub_rn(h, __fsub_rn(s, v)), __fsub_rn(p, v));
    h = s;
    l = __fadd_rn(l, __fadd_rn(t, e));
  }
  __device__ __forceinline__ void renorm() {
    const df64 s = quick_two_sum(h, l);
    h = s.hi;
    l = s.lo;
  }
  __device__ __forceinline__ df64 get() const { return df64(h, l); }
};
template <>
struct Acc<df64> {
  Dot2 re, im;
  __device__ __forceinline__ void zero() { re.h = re.l = im.h = im.l = 0.f; }
  __device__ __forceinline__ void mac(cx<df64> a, cx<df64> b) {
    re.add(a.x.hi, a.x.lo, b.x);
    re.add(-a.y.hi, -a.y.lo, b.y);
    im.add(a.x.hi, a.x.lo, b.y);
    im.add(a.y.hi, a.y.lo, b.x);
    re.renorm();
    im.renorm();
  }
  __device__ __forceinline__ cx<df64> get() const { return mk<df64>(re.get(), im.get()); }
};

// |re| + |im| in double (pivot choice, like LAPACK's izamax)
template <typename R>
__device__ __forceinline__ double cabs1(cx<R> a) {
  return fabs(to_d(a.x)) + fabs(to_d(a.y));
}
// 1/a by Smith's scaled division (no overflow for large |a|).
template <typename R>
__device__ __forceinline__ cx<R> crecip(cx<R> a) {
  if (fabs(a.x) >= fabs(a.y)) {
    R r = a.y / a.x;
    R d = a.x + a.y * r;
    return mk<R>(R(1) / d, -r / d);
  } else {
    R r = a.x / a.y;
    R d = a.x * r + a.y;
    return mk<R>(r / d, R(-1) / d);
  }
}
template <typename R>
__device__ __forceinline__ cx<R> shfl(cx<R> v, int src) {
  return mk<R>(shfl_r(v.x, src), shfl_r(v.y, src));
}

// Generic operand: pointer + leading dimension + conjugate-transpose flag.
template <typename R>
struct Op {
  const cx<R>* p;
  int ld;
  bool ct;  // true: use conj(p[c + r*ld]) as element (r,c)
  __device__ __forceinline__ cx<R> at(int r, int c) const {
    return ct ? cconj(p[c + (size_t)r * ld]) : p[r + (size_t)c * ld];
  }
};

template <typename R>
__device__ __forceinline__ Op<R> opN(const cx<R>* p, int ld) {
  Op<R> o;
  o.p = p;
  o.ld = ld;
  o.ct = false;
  return o;
}
template <typename R>
__device__ __forceinline__ Op<R> opC(const cx<R>* p, int ld) {
  Op<R> o;
  o.p = p;
  o.ld = ld;
  o.ct = true;
  return o;
}

// ---------------------------------------------------------------------------
// Epilogues: called once per output element (r,c) with the accumulated sum.
// ---------------------------------------------------------------------------
template <typename R>
struct EpiStore {  // C = s*acc
  cx<R>* c;
  int ld;
  cx<R> s;
  __device__ __forceinline__ void operator()(int r, int col, cx<R> acc) const {
    c[r + col * ld] = cmul(s, acc);
  }
};
template <typename R>
struct EpiAcc {  // C += acc
  cx<R>* c;
  int ld;
  __device__ __forceinline__ void operator()(int r, int col, cx<R> acc) const {
    c[r + col * ld] = cadd(c[r + col * ld], acc);
  }
};
template <typename R>
struct EpiAcc2 {  // C1 += acc, C2 += acc
  cx<R>* c1;
  cx<R>* c2;
  int ld;
  __device__ __forceinline__ void operator()(int r, int col, cx<R> acc) const {
    c1[r + col * ld] = cadd(c1[r + col * ld], acc);
    c2[r + col * ld] = cadd(c2[r + col * ld], acc);
  }
};
// C = z*I - H - S - acc   (H, S optional; H is an Op so it may be global)
template <typename R>
struct EpiShift {
  cx<R>* c;
  int ld;
  cx<R> z;
  Op<R> h;
  bool has_h;
  Op<R> s;
  bool has_s;
  __device__ __forceinline__ void operator()(int r, int col, cx<R> acc) const {
    cx<R> v = mk<R>(-acc.x, -acc.y);
    if (r == col) v = cadd(v, z);
    if (has_h) v = csub(v, h.at(r, col));
    if (has_s) v = csub(v, s.at(r, col));
    c[r + col * ld] = v;
  }
};

// ---------------------------------------------------------------------------
// row_gemm: C(m x n) <- epi( opA(m x k) * opB(k x n) ), one warp per row.
// S = ceil(max(k, n) / 32) register slots per lane.
// ---------------------------------------------------------------------------
template <typename R, int S, class Epi>
__device__ void row_gemm(int m, int n, int k, Op<R> A, Op<R> B, const Epi& epi) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  for (int r = warp; r < m; r += nw) {
    cx<R> arow[S];
#pragma unroll
    for (int s = 0; s < S; ++s) {
      int kk = lane + 32 * s;
      arow[s] = (kk < k) ? A.at(r, kk) : czero<R>();
    }
    Acc<R> acc[S];
#pragma unroll
    for (int t = 0; t < S; ++t) acc[t].zero();
#pragma unroll
    for (int s = 0; s < S; ++s) {
      if (32 * s < k) {
        const int kmax = min(32, k - 32 * s);
        for (int kk = 0; kk < kmax; ++kk) {
          const cx<R> a = shfl(arow[s], kk);
          const int kidx = 32 * s + kk;
#pragma unroll
          for (int t = 0; t < S; ++t) {
            const int c = lane + 32 * t;
            if (c < n) acc[t].mac(a, B.at(kidx, c));
          }
        }
      }
    }
    __syncwarp();
#pragma unroll
    for (int t = 0; t < S; ++t) {
      const int c = lane + 32 * t;
      if (c < n) epi(r, c, acc[t].get());
    }
  }
  __syncthreads();
}

// Elementwise helpers (all threads; end with a barrier).
template <typename R>
__device__ void copy_in(cx<R>* dst, int ldd, Op<R> src, int m, int n) {
  for (int i = threadIdx.x; i < m * n; i += blockDim.x) {
    const int r = i % m, c = i / m;
    dst[r + c * ldd] = src.at(r, c);
  }
  __syncthreads();
}
template <typename R>
__device__ void copy_out(cx<R>* dst, int ldd, bool conj_t, const cx<R>* src, int lds, int m, int n) {
  // dst(m x n) = src or src^H (src then n x m)
  for (int i = threadIdx.x; i < m * n; i += blockDim.x) {
    const int r = i % m, c = i / m;
    dst[r + (size_t)c * ldd] = conj_t ? cconj(src[c + r * lds]) : src[r + c * lds];
  }
  __syncthreads();
}
// dst = z*I - src
template <typename R>
__device__ void shift_neg(cx<R>* dst, int ldd, cx<R> z, const cx<R>* src, int lds, int n) {
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
    const int r = i % n, c = i / n;
    cx<R> v = src[r + c * lds];
    v = mk<R>(-v.x, -v.y);
    if (r == c) v = cadd(v, z);
    dst[r + c * ldd] = v;
  }
  __syncthreads();
}

// |a| for convergence tests: FP64 for double data, FP32 otherwise (a df64
// value's leading float carries its magnitude to ~1e-7).
__device__ __forceinline__ double abs_for_max(cx<double> e) { return hypot(e.x, e.y); }
__device__ __forceinline__ double abs_for_max(cx<float> e) { return (double)hypotf(e.x, e.y); }
__device__ __forceinline__ double abs_for_max(cx<df64> e) { return (double)hypotf(e.x.hi, e.y.hi); }

// max_ij |a_ij| (modulus), block reduction through
// `red` (>= 32 doubles).  A NaN entry makes the result NaN.
template <typename R>
__device__ double max_abs(const cx<R>* a, int ld, int m, int n, double* red) {
  double v = 0.0;
  for (int i = threadIdx.x; i < m * n; i += blockDim.x) {
    const int r = i % m, c = i / m;
    const cx<R> e = a[r + c * ld];
    const double h = abs_for_max(e);
    v = (h > v || h != h) ? h : v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w > v || w != w) ? w : v;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      const double w = __shfl_xor_sync(0xffffffffu, v, o);
      v = (w > v || w != w) ? w : v;
    }
    if (lane == 0) red[0] = v;
  }
  __syncthreads();
  v = red[0];
  __syncthreads();
  return v;
}

// Scratch vectors an inversion needs (shared memory, >= n entries each).
template <typename R>
struct InvWork {
  cx<R>* rowk;
  cx<R>* colk;
  int* perm;
  int* flag;  // single int: pivot index broadcast, then status
};

// Status bits reported per point.
enum : int {
  PF_OK = 0,
  PF_SINGULAR = 1,       // exact zero pivot (reference: ZGETRF info > 0, util.f90:44-58)
  PF_NAN = 2,            // non-finite entry (reference: ifnan stop, util.f90:29-32)
  PF_NOT_CONVERGED = 4,  // decimation hit its iteration cap
  PF_TC_TIMEOUT = 16,    // a tensor-core product's completion wait gave up (result not used)
};

// In-place inverse with explicit row exchanges (pivot rows swapped into
// place, every thread filling the pivot row and column, four barriers a
// step, the column interchanges undone one by one).  With 16 warps a CTA
// the parallel fill beats warp 0 preparing the pivot row (measured on the
// 512-thread gradient and fused mixed kernels), so inverse() uses it there.
template <typename R>
__device__ int inverse_swap(cx<R>* M, int ld, int n, InvWork<R> w) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  int status = PF_OK;
  for (int k = 0; k < n; ++k) {
    // (a) pivot search on column k, rows k..n-1 (first maximum, |re|+|im|)
    if (warp == 0) {
      double best = -1.0;
      int bi = k;
      for (int i = k + lane; i < n; i += 32) {
        const double v = cabs1(M[i + k * ld]);
        const double vv = (v != v) ? 3.0e300 : v;  // NaN wins so it gets reported
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
      if (lane == 0) w.flag[0] = bi;
    }
    __syncthreads();
    const int p = w.flag[0];
    if (tid == 0) w.perm[k] = p;
    // (b) row swap k <-> p
    if (p != k) {
      for (int j = tid; j < n; j += nt) {
        const cx<R> t = M[k + j * ld];
        M[k + j * ld] = M[p + j * ld];
        M[p + j * ld] = t;
      }
    }
    __syncthreads();
    // (c) pivot, scaled row k and column k
    const cx<R> piv = M[k + k * ld];
    if (piv.x == R(0) && piv.y == R(0)) status |= PF_SINGULAR;
    if (!(isfinite(piv.x) && isfinite(piv.y))) status |= PF_NAN;
    const cx<R> ip = crecip(piv);
    for (int j = tid; j < n; j += nt) {
      const cx<R> v = (j == k) ? ip : cmul(M[k + j * ld], ip);
      w.rowk[j] = v;
      w.colk[j] = M[j + k * ld];
    }
    __syncthreads();
    // (d) rank-1 elimination of every other row
    for (int i = tid; i < n * n; i += nt) {
      const int r = i % n, c = i / n;
      if (r == k) {
        M[r + c * ld] = w.rowk[c];
      } else if (c == k) {
        const cx<R> f = w.colk[r];
        M[r + c * ld] = mk<R>(-(f.x * ip.x - f.y * ip.y), -(f.x * ip.y + f.y * ip.x));
      } else {
        const cx<R> f = w.colk[r];
        const cx<R> rk = w.rowk[c];
        cx<R> v = M[r + c * ld];
        v.x = fma(-f.x, rk.x, fma(f.y, rk.y, v.x));
        v.y = fma(-f.x, rk.y, fma(-f.y, rk.x, v.y));
        M[r + c * ld] = v;
      }
    }
    __syncthreads();
  }
  // undo the row interchanges as column interchanges, last first
  for (int k = n - 1; k >= 0; --k) {
    const int p = w.perm[k];
    if (p != k) {
      for (int i = tid; i < n; i += nt) {
        const cx<R> t = M[i + k * ld];
        M[i + k * ld] = M[i + p * ld];
        M[i + p * ld] = t;
      }
    }
    __syncthreads();
  }
  return status;
}

// In-place inverse of the n x n matrix M (ld odd, shared memory, n <= 1024).
// Gauss-Jordan with implicit partial pivoting: the pivot of step k is the
// first maximum of |re|+|im| in column k among the rows not yet used
// (LAPACK izamax's measure); rows are never exchanged, warp 0 prepares the
// scaled pivot row and the pivot column, and every thread then updates its
// elements -- two barriers a step.  The row/column permutation is undone at
// the end by one gather: inv(k, P(j)) = M(P(k), j).
// Returns PF_OK, PF_SINGULAR or PF_NAN (uniform across the CTA).
template <typename R>
__device__ int inverse(cx<R>* M, int ld, int n, InvWork<R> w) {
  if (blockDim.x > 256) return inverse_swap(M, ld, n, w);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5;
  int status = PF_OK;
  unsigned used = 0u;  // warp 0, lane l: bit m set when row l + 32 m is pivoted
  for (int k = 0; k < n; ++k) {
    if (warp == 0) {
      double best = -1.0;
      int bi = n;
      for (int i = lane; i < n; i += 32) {
        if ((used >> (i >> 5)) & 1u) continue;
        const double v = cabs1(M[i + k * ld]);
        const double vv = (v != v) ? 3.0e300 : v;  // NaN wins so it gets reported
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
      const int p = bi;
      if ((p & 31) == lane) used |= 1u << (p >> 5);
      const cx<R> ip = crecip(M[p + k * ld]);
      for (int j = lane; j < n; j += 32) {
        w.rowk[j] = (j == k) ? ip : cmul(M[p + j * ld], ip);
        w.colk[j] = M[j + k * ld];
      }
      if (lane == 0) {
        w.perm[k] = p;
        w.flag[0] = p;
      }
    }
    __syncthreads();
    const int p = w.flag[0];
    const cx<R> piv = w.colk[p];
    if (piv.x == R(0) && piv.y == R(0)) status |= PF_SINGULAR;
    if (!(isfinite(piv.x) && isfinite(piv.y))) status |= PF_NAN;
    const cx<R> ip = w.rowk[k];
    for (int i = tid; i < n * n; i += nt) {
      const int r = i % n, c = i / n;
      if (r == p) {
        M[r + c * ld] = w.rowk[c];
      } else if (c == k) {
        const cx<R> f = w.colk[r];
        M[r + c * ld] = mk<R>(-(f.x * ip.x - f.y * ip.y), -(f.x * ip.y + f.y * ip.x));
      } else {
        const cx<R> f = w.colk[r];
        const cx<R> rk = w.rowk[c];
        cx<R> v = M[r + c * ld];
        v.x = fma(-f.x, rk.x, fma(f.y, rk.y, v.x));
        v.y = fma(-f.x, rk.y, fma(-f.y, rk.x, v.y));
        M[r + c * ld] = v;
      }
    }
    __syncthreads();
  }
  // inv(k, P(j)) = M(P(k), j), as a row gather within each column and then a
  // column scatter within each row; each pass goes through registers in
  // chunks of whole columns (rows) of at most kMaxPer elements a thread,
  // one chunk for n <= 64 with 128 or more threads.
  constexpr int kMaxPer = 32;
  cx<R> tmp[kMaxPer];
  const int per = (kMaxPer * nt) / n > 0 ? (kMaxPer * nt) / n : 1;
  for (int j0 = 0; j0 < n; j0 += per) {
    const int nc = (j0 + per < n ? j0 + per : n) - j0;
    int t = 0;
    for (int i = tid; i < n * nc; i += nt, ++t) tmp[t] = M[w.perm[i % n] + (j0 + i / n) * ld];
    __syncthreads();
    t = 0;
    for (int i = tid; i < n * nc; i += nt, ++t) M[i % n + (j0 + i / n) * ld] = tmp[t];
    __syncthreads();
  }
  for (int k0 = 0; k0 < n; k0 += per) {
    const int nrw = (k0 + per < n ? k0 + per : n) - k0;
    int t = 0;
    for (int i = tid; i < nrw * n; i += nt, ++t) tmp[t] = M[k0 + i % nrw + (i / nrw) * ld];
    __syncthreads();
    t = 0;
    for (int i = tid; i < nrw * n; i += nt, ++t) M[k0 + i % nrw + w.perm[i / nrw] * ld] = tmp[t];
    __syncthreads();
  }
  return status;
}

// Re Tr(X * Y) with X (m x n) and Y (n x m), accumulated in double,
// block reduction via `red` (>= 32 doubles).
template <typename R>
__device__ double trace_prod_re(const cx<R>* X, int ldx, Op<R> Y, int m, int n, double* red) {
  double v = 0.0;
  for (int i = threadIdx.x; i < m * n; i += blockDim.x) {
    const int r = i % m, c = i / m;
    const cx<R> a = X[r + c * ldx];
    const cx<R> b = Y.at(c, r);
    v += to_d(a.x) * to_d(b.x) - to_d(a.y) * to_d(b.y);
  }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[0] = v;
  }
  __syncthreads();
  v = red[0];
  __syncthreads();
  return v;
}

}  // namespace pf
