/*
 * C restatement of the transmission oracle (test infrastructure and CPU
 * baseline only; never part of the product): the left advanced and right
 * retarded Lopez-Sancho decimations of negf/surface.f90:479-568, the
 * left-to-right RGF sweep with the right-lead closure of
 * negf/lesser.f90:547-654 and the Caroli trace T_L of lesser.f90:787-800,
 * for a batch of energies of one q, one point per OpenMP iteration.
 *
 * It follows oracle/negf.py (the numpy restatement) step for step; the
 * blocks come in the layout of the C ABI: interleaved complex128,
 * column-major, Hd [L][n x n], Hdv [L-1][n x n], Hld n_l x n, Hrd n_r x n.
 * Dense inverses are Gauss-Jordan with partial pivoting.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cz;

#define AT(M, ld, r, c) ((M)[(size_t)(c) * (ld) + (r)])

/* C = A (m x k) * B (k x p); ops: 'N' or 'C' (conjugate transpose) on the
 * stored matrix; all column-major with the given leading dimensions. */
static void gemm(int m, int p, int k, const cz* A, int lda, char ta, const cz* B, int ldb, char tb, cz* C,
                 int ldc) {
  for (int j = 0; j < p; ++j)
    for (int i = 0; i < m; ++i) AT(C, ldc, i, j) = 0;
  for (int j = 0; j < p; ++j) {
    for (int l = 0; l < k; ++l) {
      const cz b = (tb == 'N') ? AT(B, ldb, l, j) : conj(AT(B, ldb, j, l));
      if (b == 0) continue;
      if (ta == 'N') {
        const cz* a = &AT(A, lda, 0, l);
        cz* c = &AT(C, ldc, 0, j);
        for (int i = 0; i < m; ++i) c[i] += a[i] * b;
      } else {
        for (int i = 0; i < m; ++i) AT(C, ldc, i, j) += conj(AT(A, lda, l, i)) * b;
      }
    }
  }
}

/* In-place inverse of the n x n matrix A (ld n); returns 1 when singular. */
static int inverse(int n, cz* A, cz* work, int* piv) {
  /* Gauss-Jordan on [A | I] with row pivoting, stored as A and work */
  cz* Inv = work;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) AT(Inv, n, i, j) = (i == j) ? 1.0 : 0.0;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = cabs(AT(A, n, k, k));
    for (int i = k + 1; i < n; ++i) {
      const double v = cabs(AT(A, n, i, k));
      if (v > best) {
        best = v;
        p = i;
      }
    }
    piv[k] = p;
    if (best == 0.0) return 1;
    if (p != k) {
      for (int j = 0; j < n; ++j) {
        cz t = AT(A, n, k, j);
        AT(A, n, k, j) = AT(A, n, p, j);
        AT(A, n, p, j) = t;
        t = AT(Inv, n, k, j);
        AT(Inv, n, k, j) = AT(Inv, n, p, j);
        AT(Inv, n, p, j) = t;
      }
    }
    const cz d = 1.0 / AT(A, n, k, k);
    for (int j = 0; j < n; ++j) {
      AT(A, n, k, j) *= d;
      AT(Inv, n, k, j) *= d;
    }
    for (int i = 0; i < n; ++i) {
      if (i == k) continue;
      const cz f = AT(A, n, i, k);
      if (f == 0) continue;
      for (int j = 0; j < n; ++j) {
        AT(A, n, i, j) -= f * AT(A, n, k, j);
        AT(Inv, n, i, j) -= f * AT(Inv, n, k, j);
      }
    }
  }
  memcpy(A, Inv, sizeof(cz) * (size_t)n * n);
  return 0;
}

/* Lopez-Sancho decimation (negf/surface.f90:488-497): g = inv(z - es). */
static int decimate(int n, cz z, const cz* H00, const cz* alpha0, char ta, const cz* beta0, char tb,
                    double convergence, int max_iter, cz* g, int* iters, cz* s) {
  const size_t nn = (size_t)n * n;
  cz *e1 = s, *es = s + nn, *al = s + 2 * nn, *be = s + 3 * nn, *ive = s + 4 * nn, *ai = s + 5 * nn,
     *bi = s + 6 * nn, *t = s + 7 * nn, *w = s + 8 * nn;
  int* piv = (int*)(s + 9 * nn);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      AT(e1, n, i, j) = AT(H00, n, i, j);
      AT(al, n, i, j) = (ta == 'N') ? AT(alpha0, n, i, j) : conj(AT(alpha0, n, j, i));
      AT(be, n, i, j) = (tb == 'N') ? AT(beta0, n, i, j) : conj(AT(beta0, n, j, i));
    }
  memcpy(es, e1, sizeof(cz) * nn);
  int it = 0, bad = 0;
  for (;;) {
    double amax = 0.0;
    for (size_t q = 0; q < nn; ++q) amax = fmax(amax, cabs(al[q]));
    if (!(amax > convergence) || it >= max_iter) break;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) AT(ive, n, i, j) = (i == j ? z : 0.0) - AT(e1, n, i, j);
    bad |= inverse(n, ive, w, piv);
    gemm(n, n, n, al, n, 'N', ive, n, 'N', ai, n);  /* alpha ive */
    gemm(n, n, n, be, n, 'N', ive, n, 'N', bi, n);  /* beta ive */
    gemm(n, n, n, ai, n, 'N', be, n, 'N', t, n);    /* alpha ive beta */
    for (size_t q = 0; q < nn; ++q) {
      e1[q] += t[q];
      es[q] += t[q];
    }
    gemm(n, n, n, bi, n, 'N', al, n, 'N', t, n);    /* beta ive alpha */
    for (size_t q = 0; q < nn; ++q) e1[q] += t[q];
    gemm(n, n, n, ai, n, 'N', al, n, 'N', t, n);
    memcpy(al, t, sizeof(cz) * nn);
    gemm(n, n, n, bi, n, 'N', be, n, 'N', t, n);
    memcpy(be, t, sizeof(cz) * nn);
    ++it;
  }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) AT(g, n, i, j) = (i == j ? z : 0.0) - AT(es, n, i, j);
  bad |= inverse(n, g, w, piv);
  *iters = it;
  return bad;
}

/* Scratch for one point, in complex numbers. */
size_t oracle_c_scratch(int n, int nl, int nr) {
  int m = n > nl ? n : nl;
  m = m > nr ? m : nr;
  return (size_t)24 * m * m + (size_t)m;  /* 9 decimation + piv + sweep matrices */
}

/*
 * T_L of npts energies of one q (columns-major blocks as the C ABI takes
 * them).  Returns the number of points whose inverses hit a zero pivot.
 */
int oracle_c_transport(int n, int nl, int nr, int L, const double* HL_, const double* HLv_, const double* HR_,
                       const double* HRv_, const double* Hd_, const double* Hdv_, const double* Hld_,
                       const double* Hrd_, int npts, const double* E, double eta, double eta0,
                       double dev_factor, double convergence, int max_iter, double* transl, int* iters) {
  const cz* HL = (const cz*)HL_;
  const cz* HLv = (const cz*)HLv_;
  const cz* HR = (const cz*)HR_;
  const cz* HRv = (const cz*)HRv_;
  const cz* Hd = (const cz*)Hd_;
  const cz* Hdv = (const cz*)Hdv_;
  const cz* Hld = (const cz*)Hld_;
  const cz* Hrd = (const cz*)Hrd_;
  int m = n > nl ? n : nl;
  m = m > nr ? m : nr;
  const size_t mm = (size_t)m * m;
  int nbad = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : nbad)
  for (int p = 0; p < npts; ++p) {
    cz* S = (cz*)malloc(sizeof(cz) * oracle_c_scratch(n, nl, nr));
    cz *gl = S + 10 * mm, *gr = S + 11 * mm, *T1 = S + 12 * mm, *T2 = S + 13 * mm, *g = S + 14 * mm,
       *G0N = S + 15 * mm, *A = S + 16 * mm, *sr = S + 17 * mm, *gml = S + 18 * mm, *gmr = S + 19 * mm,
       *W = S + 20 * mm;
    int* piv = (int*)(S + 21 * mm);
    int bad = 0, itl = 0, itr = 0;
    const double eps = E[p] * eta + eta0;
    /* left, advanced: z = E - i eps, alpha = HLv^H, beta = HLv */
    bad |= decimate(nl, E[p] - I * eps, HL, HLv, 'C', HLv, 'N', convergence, max_iter, gl, &itl, S);
    /* sl_adv = HLv^H gl_adv HLv; gml_adv = i (sl - sl^H); the wrapper takes
     * gl = gl_adv^H, gml = -gml_adv */
    gemm(nl, nl, nl, HLv, nl, 'C', gl, nl, 'N', T1, nl);
    gemm(nl, nl, nl, T1, nl, 'N', HLv, nl, 'N', T2, nl);
    for (int j = 0; j < nl; ++j)
      for (int i = 0; i < nl; ++i) AT(gml, nl, i, j) = -(I * (AT(T2, nl, i, j) - conj(AT(T2, nl, j, i))));
    for (int j = 0; j < nl; ++j)
      for (int i = 0; i < nl; ++i) AT(T1, nl, i, j) = conj(AT(gl, nl, j, i));
    memcpy(gl, T1, sizeof(cz) * (size_t)nl * nl);
    /* right, retarded: z = E + i eps, alpha = HRv^H, beta = HRv */
    bad |= decimate(nr, E[p] + I * eps, HR, HRv, 'C', HRv, 'N', convergence, max_iter, gr, &itr, S);
    gemm(nr, nr, nr, HRv, nr, 'C', gr, nr, 'N', T1, nr);
    gemm(nr, nr, nr, T1, nr, 'N', HRv, nr, 'N', sr, nr);
    for (int j = 0; j < nr; ++j)
      for (int i = 0; i < nr; ++i) AT(gmr, nr, i, j) = I * (AT(sr, nr, i, j) - conj(AT(sr, nr, j, i)));
    /* left-to-right sweep: g_1 = inv(zD - Hd_1 - Hld^H gl Hld), G0N = gl Hld g_1 */
    const cz zD = E[p] + I * dev_factor * eps;
    gemm(nl, n, nl, gl, nl, 'N', Hld, nl, 'N', T1, nl);          /* gl Hld (nl x n) */
    gemm(n, n, nl, Hld, nl, 'C', T1, nl, 'N', A, n);             /* Hld^H gl Hld */
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) AT(g, n, i, j) = (i == j ? zD : 0.0) - AT(Hd, n, i, j) - AT(A, n, i, j);
    bad |= inverse(n, g, W, piv);
    gemm(nl, n, n, T1, nl, 'N', g, n, 'N', G0N, nl);              /* G0N = gl Hld g */
    for (int l = 1; l < L; ++l) {
      const cz* V = Hdv + (size_t)(l - 1) * n * n;
      const cz* Hl = Hd + (size_t)l * n * n;
      gemm(n, n, n, g, n, 'N', V, n, 'N', T1, n);                 /* g V */
      gemm(n, n, n, V, n, 'C', T1, n, 'N', A, n);                 /* V^H g V */
      gemm(nl, n, n, G0N, nl, 'N', V, n, 'N', T2, nl);            /* G0N V */
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) AT(g, n, i, j) = (i == j ? zD : 0.0) - AT(Hl, n, i, j) - AT(A, n, i, j);
      bad |= inverse(n, g, W, piv);
      gemm(nl, n, n, T2, nl, 'N', g, n, 'N', G0N, nl);
    }
    /* right lead block: GRR = inv(zD - HR - sr - V^H g V), V = Hrd^H (n x nr) */
    gemm(n, nr, n, g, n, 'N', Hrd, nr, 'C', T1, n);               /* g V */
    gemm(nr, nr, n, Hrd, nr, 'N', T1, n, 'N', A, nr);             /* V^H g V = Hrd g Hrd^H */
    for (int j = 0; j < nr; ++j)
      for (int i = 0; i < nr; ++i)
        AT(A, nr, i, j) = (i == j ? zD : 0.0) - AT(HR, nr, i, j) - AT(sr, nr, i, j) - AT(A, nr, i, j);
    bad |= inverse(nr, A, W, piv);
    gemm(nl, nr, n, G0N, nl, 'N', Hrd, nr, 'C', T1, nl);          /* G0N V */
    gemm(nl, nr, nr, T1, nl, 'N', A, nr, 'N', T2, nl);            /* G_D_LR = G0N V GRR (nl x nr) */
    /* Caroli: T_L = Re Tr[(G_D_LR gmr)(G_D_LR^H gml)] */
    gemm(nl, nr, nr, T2, nl, 'N', gmr, nr, 'N', T1, nl);          /* P (nl x nr) */
    gemm(nr, nl, nl, T2, nl, 'C', gml, nl, 'N', A, nr);           /* Q (nr x nl) */
    double tr = 0.0;
    for (int i = 0; i < nl; ++i)
      for (int k = 0; k < nr; ++k) tr += creal(AT(T1, nl, i, k) * AT(A, nr, k, i));
    transl[p] = tr < 1.0e-60 ? 0.0 : tr;
    if (iters) iters[p] = itl;
    nbad += bad ? 1 : 0;
    free(S);
  }
  return nbad;
}

/* Threads of the OpenMP loop over energies (no-op without OpenMP). */
int oracle_c_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  return omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}
