// Mode-resolved transmission (negf/velocity_mat.f90:1692-3148), FP64.
//
// One CTA per lead eigenproblem.  The dense kernels work on column-major
// shared-memory matrices with the odd leading dimension of cmat.cuh:
//   schur       : complex Schur form A = Z T Z^H.  Householder reduction to
//                 upper Hessenberg form, then single-shift implicit QR with
//                 Wilkinson shifts and Givens rotations (the textbook
//                 algorithm, e.g. Golub & Van Loan 7.4-7.5), T and Z kept in
//                 full (the role of ZGEES / ZHSEQR in util.f90:226-262,
//                 359-454).
//   tri_eigvecs : eigenvectors of the triangular T by back substitution with
//                 the small-denominator guard of ZTREVC, then U = Z Y and
//                 the ZGEEV normalisation (unit 2-norm, largest |u_k|^2
//                 component made real and positive).
//   sqrt_tri    : principal square root of an upper-triangular T by the
//                 super-diagonal recurrence of util.f90:411-429 (zero when
//                 the denominator U_ii + U_jj vanishes).
#pragma once
#include "cmat.cuh"

namespace pf {
namespace modes {

using C = cx<double>;

enum : int { PF_EIG_NOT_CONVERGED = 8 };

__device__ __forceinline__ double cab(C a) { return fabs(a.x) + fabs(a.y); }
__device__ __forceinline__ C cscale(C a, double s) { return mk<double>(a.x * s, a.y * s); }
__device__ __forceinline__ C cdiv(C a, C b) { return cmul(a, crecip(b)); }
__device__ __forceinline__ C csqrt_p(C a) {
  // principal square root (branch cut on the negative real axis)
  const double r = hypot(a.x, a.y);
  if (r == 0.0) return mk<double>(0.0, 0.0);
  double re = sqrt(0.5 * (r + fabs(a.x)));
  double im = a.y / (2.0 * re);
  if (a.x >= 0.0) return mk<double>(re, im);
  return mk<double>(fabs(im), a.y >= 0.0 ? re : -re);
}

// Sum over the CTA (red >= 32 doubles); all threads get the result.
__device__ __forceinline__ double block_sum(double v, double* red) {
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
__device__ __forceinline__ C block_csum(C v, double* red) {
  const double a = block_sum(v.x, red);
  const double b = block_sum(v.y, red);
  return mk<double>(a, b);
}

// Wilkinson shift: the eigenvalue of [[a b][c d]] closer to d.
__device__ __forceinline__ C wilkinson(C a, C b, C c, C d) {
  const C t = cscale(csub(a, d), 0.5);
  C s = csqrt_p(cfma(t, t, cmul(b, c)));
  if (t.x * s.x + t.y * s.y < 0.0) s = mk<double>(-s.x, -s.y);
  const C den = cadd(t, s);
  if (den.x == 0.0 && den.y == 0.0) return d;
  return csub(d, cdiv(cmul(b, c), den));
}

// Givens pair (c real, s complex) with [c s; -conj(s) c] [x; y] = [r; 0].
__device__ __forceinline__ void givens(C x, C y, double* c, C* s, C* r) {
  const double ax = hypot(x.x, x.y), ay = hypot(y.x, y.y);
  if (ay == 0.0) {
    *c = 1.0;
    *s = mk<double>(0.0, 0.0);
    *r = x;
    return;
  }
  if (ax == 0.0) {
    *c = 0.0;
    *s = mk<double>(1.0, 0.0);
    *r = y;
    return;
  }
  const double nrm = hypot(ax, ay);
  const C ph = cscale(x, 1.0 / ax);  // x / |x|
  *c = ax / nrm;
  *s = cscale(cmul(ph, cconj(y)), 1.0 / nrm);
  *r = cscale(ph, nrm);
}

// In-place complex Schur form of A (n x n, shared, ld): on return A holds T
// (upper triangular) and Z the unitary Schur vectors.  v (>= n entries) is
// shared scratch.  Returns PF_OK or PF_EIG_NOT_CONVERGED.
__device__ int schur(C* A, C* Z, int ld, int n, C* v, double* red) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < n * n; i += nt) {
    const int r = i % n, c = i / n;
    Z[r + c * ld] = mk<double>(r == c ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  // ---- Householder reduction to upper Hessenberg form
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1;  // length of x = A[k+1:n, k]
    double part = 0.0;
    for (int i = tid; i < m; i += nt) {
      const C e = A[(k + 1 + i) + k * ld];
      part += e.x * e.x + e.y * e.y;
    }
    const double xn2 = block_sum(part, red);
    const C x0 = A[(k + 1) + k * ld];
    const double x0a = hypot(x0.x, x0.y);
    const double tail = xn2 - x0a * x0a;
    if (!(tail > 0.0)) continue;  // already reduced
    const double xn = sqrt(xn2);
    const C ph = x0a > 0.0 ? cscale(x0, 1.0 / x0a) : mk<double>(1.0, 0.0);
    const C alpha = cscale(ph, -xn);  // P x = alpha e1
    for (int i = tid; i < m; i += nt) v[i] = (i == 0) ? csub(x0, alpha) : A[(k + 1 + i) + k * ld];
    __syncthreads();
    // v^H v = |x0 - alpha|^2 + tail
    const C v0 = csub(x0, alpha);
    const double beta = 2.0 / (v0.x * v0.x + v0.y * v0.y + tail);
    // left: A[k+1:, j] -= beta v (v^H A[k+1:, j]) for j >= k
    for (int j = k + tid; j < n; j += nt) {
      C w = mk<double>(0.0, 0.0);
      for (int i = 0; i < m; ++i) w = cfma(cconj(v[i]), A[(k + 1 + i) + j * ld], w);
      w = cscale(w, beta);
      for (int i = 0; i < m; ++i) A[(k + 1 + i) + j * ld] = csub(A[(k + 1 + i) + j * ld], cmul(v[i], w));
    }
    __syncthreads();
    // right: A[i, k+1:] -= beta (A[i, k+1:] v) v^H for all rows; same on Z
    for (int t = tid; t < 2 * n; t += nt) {
      C* M = t < n ? A : Z;
      const int i = t < n ? t : t - n;
      C u = mk<double>(0.0, 0.0);
      for (int j = 0; j < m; ++j) u = cfma(M[i + (k + 1 + j) * ld], v[j], u);
      u = cscale(u, beta);
      for (int j = 0; j < m; ++j) M[i + (k + 1 + j) * ld] = csub(M[i + (k + 1 + j) * ld], cmul(u, cconj(v[j])));
    }
    __syncthreads();
    if (tid == 0) {
      A[(k + 1) + k * ld] = alpha;
      for (int i = 2; i <= m; ++i) A[(k + i) + k * ld] = mk<double>(0.0, 0.0);
    }
    __syncthreads();
  }
  // ---- shifted QR on the Hessenberg matrix
  const double ulp = 2.220446049250313e-16;
  const double smlnum = 1.0e-290;
  int hi = n - 1;
  int its = 0, total = 0;
  const int max_total = 30 * (n > 10 ? n : 10);
  int status = PF_OK;
  while (hi > 0) {
    // deflation: find the start l of the unreduced block ending at hi
    int l = hi;
    while (l > 0) {
      const C s = A[l + (l - 1) * ld];
      const double tst = cab(A[(l - 1) + (l - 1) * ld]) + cab(A[l + l * ld]);
      if (cab(s) <= fmax(ulp * tst, smlnum)) break;
      --l;
    }
    __syncthreads();
    if (l > 0) {
      if (tid == 0) A[l + (l - 1) * ld] = mk<double>(0.0, 0.0);
      __syncthreads();
    }
    if (l == hi) {
      --hi;
      its = 0;
      continue;
    }
    if (total >= max_total) {
      status = PF_EIG_NOT_CONVERGED;
      break;
    }
    ++its;
    ++total;
    C mu;
    if (its % 10 == 0) {
      const C d = A[hi + hi * ld];
      mu = mk<double>(d.x + 0.75 * cab(A[hi + (hi - 1) * ld]), d.y);
    } else {
      mu = wilkinson(A[(hi - 1) + (hi - 1) * ld], A[(hi - 1) + hi * ld], A[hi + (hi - 1) * ld], A[hi + hi * ld]);
    }
    for (int k = l; k < hi; ++k) {
      C x, y;
      if (k == l) {
        x = csub(A[l + l * ld], mu);
        y = A[(l + 1) + l * ld];
      } else {
        x = A[k + (k - 1) * ld];
        y = A[(k + 1) + (k - 1) * ld];
      }
      double c;
      C s, r;
      givens(x, y, &c, &s, &r);
      __syncthreads();
      // rows k, k+1: [c s; -conj(s) c] applied on columns j >= jl
      const int jl = (k == l) ? l : k - 1;
      for (int j = jl + tid; j < n; j += nt) {
        const C a = A[k + j * ld], b = A[(k + 1) + j * ld];
        A[k + j * ld] = cadd(cscale(a, c), cmul(s, b));
        A[(k + 1) + j * ld] = csub(cscale(b, c), cmul(cconj(s), a));
      }
      __syncthreads();
      if (k > l && tid == 0) {
        A[k + (k - 1) * ld] = r;
        A[(k + 1) + (k - 1) * ld] = mk<double>(0.0, 0.0);
      }
      // columns k, k+1 times [c -s; conj(s) c]^T... i.e. M <- M R^H:
      //   col_k' = c col_k + conj(s) col_{k+1},  col_{k+1}' = -s col_k + c col_{k+1}
      const int ilast = (k + 2 < hi) ? k + 2 : hi;
      for (int t = tid; t < (ilast + 1) + n; t += nt) {
        C* M = t <= ilast ? A : Z;
        const int i = t <= ilast ? t : t - (ilast + 1);
        const C a = M[i + k * ld], b = M[i + (k + 1) * ld];
        M[i + k * ld] = cadd(cscale(a, c), cmul(cconj(s), b));
        M[i + (k + 1) * ld] = csub(cscale(b, c), cmul(s, a));
      }
      __syncthreads();
    }
  }
  // clean the strictly lower part
  for (int i = tid; i < n * n; i += nt) {
    const int r = i % n, c = i / n;
    if (r > c) A[r + c * ld] = mk<double>(0.0, 0.0);
  }
  __syncthreads();
  return status;
}

// Eigenvectors of the upper-triangular T (back substitution, one thread per
// eigenvector) into Y (upper triangular, column i for eigenvalue T_ii).
__device__ void tri_eigvecs(const C* T, C* Y, int ld, int n) {
  const double ulp = 2.220446049250313e-16;
  const double smlnum = 1.0e-290;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const C lam = T[i + i * ld];
    const double smin = fmax(ulp * cab(lam), smlnum);
    for (int k = i + 1; k < n; ++k) Y[k + i * ld] = mk<double>(0.0, 0.0);
    Y[i + i * ld] = mk<double>(1.0, 0.0);
    for (int k = i - 1; k >= 0; --k) {
      C acc = mk<double>(0.0, 0.0);
      for (int j = k + 1; j <= i; ++j) acc = cfma(T[k + j * ld], Y[j + i * ld], acc);
      C d = csub(T[k + k * ld], lam);
      if (cab(d) < smin) d = mk<double>(smin, 0.0);
      C yk = cdiv(acc, d);
      Y[k + i * ld] = mk<double>(-yk.x, -yk.y);
      // keep the partial vector bounded
      const double big = cab(Y[k + i * ld]);
      if (big > 1.0e100) {
        const double sc = 1.0 / big;
        for (int j = k; j <= i; ++j) Y[j + i * ld] = cscale(Y[j + i * ld], sc);
      }
    }
  }
  __syncthreads();
}

// ZGEEV normalisation of the columns of U: unit 2-norm, then the first
// component of largest re^2 + im^2 rotated to be real and positive.
__device__ void normalise_columns(C* U, int ld, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double s = 0.0;
    for (int r = 0; r < n; ++r) {
      const C e = U[r + i * ld];
      s += e.x * e.x + e.y * e.y;
    }
    const double inv = s > 0.0 ? 1.0 / sqrt(s) : 0.0;
    double best = -1.0;
    int kb = 0;
    for (int r = 0; r < n; ++r) {
      const C e = cscale(U[r + i * ld], inv);
      U[r + i * ld] = e;
      const double m = e.x * e.x + e.y * e.y;
      if (m > best) {
        best = m;
        kb = r;
      }
    }
    const C e = U[kb + i * ld];
    const double a = sqrt(best);
    if (a > 0.0) {
      const C ph = cscale(cconj(e), 1.0 / a);
      for (int r = 0; r < n; ++r) U[r + i * ld] = cmul(U[r + i * ld], ph);
      U[kb + i * ld].y = 0.0;
    }
  }
  __syncthreads();
}

// Principal square root of upper-triangular S into Usq (util.f90:411-429).
__device__ void sqrt_tri(const C* S, C* Usq, int ld, int n) {
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
    const int r = i % n, c = i / n;
    Usq[r + c * ld] = (r == c) ? csqrt_p(S[r + c * ld]) : mk<double>(0.0, 0.0);
  }
  __syncthreads();
  for (int sd = 1; sd < n; ++sd) {
    for (int i = threadIdx.x; i < n - sd; i += blockDim.x) {
      const int j = i + sd;
      C u = S[i + j * ld];
      for (int k = i + 1; k < j; ++k) u = csub(u, cmul(Usq[i + k * ld], Usq[k + j * ld]));
      const C den = cadd(Usq[i + i * ld], Usq[j + j * ld]);
      Usq[i + j * ld] = (den.x != 0.0 || den.y != 0.0) ? cdiv(u, den) : mk<double>(0.0, 0.0);
    }
    __syncthreads();
  }
}

// The quirky Gram-Schmidt of util.f90:800-823 on the columns `cols[0..p)`
// of U: coefficient dot_product(U1_i, U2_j) / dot_product(U2_j, U2_j), with
// Fortran's dot_product conjugating its first argument (U1 = the columns
// before the loop, kept in O).  Normalised at the end.
__device__ void gram_schmidt_cols(C* U, C* O, int ld, int n, const int* cols, int p, double* red) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int t = tid; t < n * p; t += nt) {
    const int r = t % n, q = t / n;
    O[r + q * ld] = U[r + cols[q] * ld];
  }
  __syncthreads();
  for (int i = 1; i < p; ++i) {
    const int ci = cols[i];
    for (int j = 0; j < i; ++j) {
      const int cj = cols[j];
      C num = mk<double>(0.0, 0.0);
      double den = 0.0;
      for (int r = tid; r < n; r += nt) {
        const C a = O[r + i * ld];      // U1(:, i)
        const C b = U[r + cj * ld];     // U2(:, j)
        num = cfma(cconj(a), b, num);
        den += b.x * b.x + b.y * b.y;
      }
      num = block_csum(num, red);
      den = block_sum(den, red);
      const C coef = cscale(num, 1.0 / den);
      for (int r = tid; r < n; r += nt) U[r + ci * ld] = csub(U[r + ci * ld], cmul(coef, U[r + cj * ld]));
      __syncthreads();
    }
  }
  for (int q = 0; q < p; ++q) {
    const int cq = cols[q];
    double s = 0.0;
    for (int r = tid; r < n; r += nt) {
      const C b = U[r + cq * ld];
      s += b.x * b.x + b.y * b.y;
    }
    s = block_sum(s, red);
    const double inv = 1.0 / sqrt(s);
    for (int r = tid; r < n; r += nt) U[r + cq * ld] = cscale(U[r + cq * ld], inv);
    __syncthreads();
  }
}

}  // namespace modes
}  // namespace pf
