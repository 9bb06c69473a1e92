// Tight-binding H(k) blocks (tb/hamiltonian.f90:444-519 gen_ham with the
// Slater-Koster table V_sk, :74-417, the power law V_term, :28-55, and the
// onsite rule, :57-72), built directly as the block-tridiagonal pieces the
// transport entries take: for layers I (atom ranges) the diagonal blocks
// H_{I,I} and the upper couplings H_{I,I+1} of the Hermitised matrix
// 0.5 (H + H^H) (tb/util.f90:709-718).  One thread per output element and
// k; every element sums the 27 cell images in the reference's order.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include <vector>

#include "../../include/phinfortran_gb300.h"

namespace {

thread_local char g_err[512] = "";
int set_err(int code, const char* msg) {
  snprintf(g_err, sizeof(g_err), "%s", msg);
  return code;
}

constexpr double kAng = 1.0e-10;
// Fortran sqrt(3.0): a single-precision literal, promoted to double
__device__ __forceinline__ double s3() { return (double)sqrtf(3.0f); }

struct TbArgs {
  int nspecies;
  const double* V;    // [si][sj][n1][n2][t], 4x4x4 per species pair
  const double* Vn;
  const double* r_d;  // [si][sj]
  const double* pos;  // [natoms][3]
  const int* oatom;   // per orbital: atom
  const int* ospec;   // per orbital: species
  const int* ocode;   // per orbital: 0 s .. 8 dz2, 9 s*
  double lat[9];      // rows = lattice vectors
  double rcut;
};

__device__ __forceinline__ int principal(int o) { return o == 0 ? 1 : (o <= 3 ? 2 : (o <= 8 ? 3 : 4)); }

__device__ __forceinline__ double vterm(const TbArgs& a, int i, int j, int n1, int n2, int t, double dist) {
  const size_t idx = ((((size_t)i * a.nspecies + j) * 4 + (n1 - 1)) * 4 + (n2 - 1)) * 4 + (t - 1);
  const double d0 = a.r_d[(size_t)i * a.nspecies + j];
  return a.V[idx] * pow(d0 / dist / kAng, a.Vn[idx]);
}

__device__ double onsite(const TbArgs& a, int i, int j, int o1, int o2) {
  if (o1 != o2) return 0.0;
  const int n = principal(o1);
  const size_t idx = ((((size_t)i * a.nspecies + j) * 4 + (n - 1)) * 4 + (n - 1)) * 4;
  return a.V[idx];
}

// Slater-Koster element (orbital codes o1 on species i, o2 on species j).
__device__ double vsk(const TbArgs& a, int i, int j, int o1, int o2, double rx, double ry, double rz) {
  const double dist = sqrt(rx * rx + ry * ry + rz * rz);
  const double l = rx / dist, m = ry / dist, n = rz / dist;
  const double l2 = l * l, m2 = m * m, n2 = n * n;
  const double S3 = s3();
#define T(a_, b_, p1, p2, t) vterm(a, a_, b_, p1, p2, t, dist)
  switch (o1 * 10 + o2) {
    case 0: return T(i, j, 1, 1, 2);                                   // s s
    case 1: return l * T(i, j, 1, 2, 2);                               // s px
    case 10: return -l * T(j, i, 1, 2, 2);                             // px s
    case 2: return m * T(i, j, 1, 2, 2);                               // s py
    case 20: return -m * T(j, i, 1, 2, 2);
    case 3: return n * T(i, j, 1, 2, 2);                               // s pz
    case 30: return -n * T(j, i, 1, 2, 2);
    case 11: return l2 * T(i, j, 2, 2, 2) + (1 - l2) * T(i, j, 2, 2, 3);  // px px
    case 22: return m2 * T(i, j, 2, 2, 2) + (1 - m2) * T(i, j, 2, 2, 3);
    case 33: return n2 * T(i, j, 2, 2, 2) + (1 - n2) * T(i, j, 2, 2, 3);
    case 12: case 21: return l * m * T(i, j, 2, 2, 2) - l * m * T(i, j, 2, 2, 3);
    case 23: case 32: return m * n * T(i, j, 2, 2, 2) - m * n * T(i, j, 2, 2, 3);
    case 13: case 31: return l * n * T(i, j, 2, 2, 2) - l * n * T(i, j, 2, 2, 3);
    // s - d
    case 4: return S3 * (l * m) * T(i, j, 1, 3, 2);
    case 40: return S3 * (l * m) * T(j, i, 1, 3, 2);
    case 5: return S3 * (m * n) * T(i, j, 1, 3, 2);
    case 50: return S3 * (m * n) * T(j, i, 1, 3, 2);
    case 6: return S3 * (l * n) * T(i, j, 1, 3, 2);
    case 60: return S3 * (l * n) * T(j, i, 1, 3, 2);
    case 7: return (S3 / 2) * (l2 - m2) * T(i, j, 1, 3, 2);
    case 70: return (S3 / 2) * (l2 - m2) * T(j, i, 1, 3, 2);
    case 8: return (n2 - (l2 + m2) / 2) * T(i, j, 1, 3, 2);
    case 80: return (n2 - (l2 + m2) / 2) * T(j, i, 1, 3, 2);
    // px - d
    case 14: return S3 * (l2 * m) * T(i, j, 2, 3, 2) + m * (1 - 2 * l2) * T(i, j, 2, 3, 3);
    case 41: return -S3 * (l2 * m) * T(j, i, 2, 3, 2) - m * (1 - 2 * l2) * T(j, i, 2, 3, 3);
    case 15: return S3 * (l * m * n) * T(i, j, 2, 3, 2) - 2 * (l * m * n) * T(i, j, 2, 3, 3);
    case 51: return -S3 * (l * m * n) * T(j, i, 2, 3, 2) + 2 * (l * m * n) * T(j, i, 2, 3, 3);
    case 16: return S3 * (l2 * n) * T(i, j, 2, 3, 2) + n * (1 - 2 * l2) * T(i, j, 2, 3, 3);
    case 61: return -S3 * (l2 * n) * T(j, i, 2, 3, 2) - n * (1 - 2 * l2) * T(j, i, 2, 3, 3);
    // py - d
    case 24: return S3 * (m2 * l) * T(i, j, 2, 3, 2) + l * (1 - 2 * m2) * T(i, j, 2, 3, 3);
    case 42: return -S3 * (m2 * l) * T(j, i, 2, 3, 2) - l * (1 - 2 * m2) * T(j, i, 2, 3, 3);
    case 25: return S3 * (m2 * n) * T(i, j, 2, 3, 2) + n * (1 - 2 * m2) * T(i, j, 2, 3, 3);
    case 52: return -S3 * (m2 * n) * T(j, i, 2, 3, 2) - n * (1 - 2 * m2) * T(j, i, 2, 3, 3);
    case 26: return S3 * (l * m * n) * T(i, j, 2, 3, 2) - 2 * (l * m * n) * T(i, j, 2, 3, 3);
    case 62: return -S3 * (l * m * n) * T(j, i, 2, 3, 2) + 2 * (l * m * n) * T(j, i, 2, 3, 3);
    // pz - d
    case 34: return S3 * (l * m * n) * T(i, j, 2, 3, 2) - 2 * (l * m * n) * T(i, j, 2, 3, 3);
    case 43: return -S3 * (l * m * n) * T(j, i, 2, 3, 2) + 2 * (l * m * n) * T(j, i, 2, 3, 3);
    case 35: return S3 * (n2 * m) * T(i, j, 2, 3, 2) + m * (1 - 2 * n2) * T(i, j, 2, 3, 3);
    case 53: return -S3 * (n2 * m) * T(j, i, 2, 3, 2) - m * (1 - 2 * n2) * T(j, i, 2, 3, 3);
    case 36: return S3 * (n2 * l) * T(i, j, 2, 3, 2) + l * (1 - 2 * n2) * T(i, j, 2, 3, 3);
    case 63: return -S3 * (n2 * l) * T(j, i, 2, 3, 2) - l * (1 - 2 * n2) * T(j, i, 2, 3, 3);
    // p - dx2-y2
    case 17: return (S3 / 2) * l * (l2 - m2) * T(i, j, 2, 3, 2) + l * (1 - l2 + m2) * T(i, j, 2, 3, 3);
    case 71: return -(S3 / 2) * l * (l2 - m2) * T(j, i, 2, 3, 2) - l * (1 - l2 + m2) * T(j, i, 2, 3, 3);
    case 27: return (S3 / 2) * m * (l2 - m2) * T(i, j, 2, 3, 2) - m * (1 + l2 - m2) * T(i, j, 2, 3, 3);
    case 72: return -(S3 / 2) * m * (l2 - m2) * T(j, i, 2, 3, 2) + m * (1 + l2 - m2) * T(j, i, 2, 3, 3);
    case 37: return (S3 / 2) * n * (l2 - m2) * T(i, j, 2, 3, 2) - n * (l2 - m2) * T(i, j, 2, 3, 3);
    case 73: return -(S3 / 2) * n * (l2 - m2) * T(j, i, 2, 3, 2) + n * (l2 - m2) * T(j, i, 2, 3, 3);
    // p - dz2
    case 18: return l * (n2 - (l2 + m2) / 2) * T(i, j, 2, 3, 2) - S3 * l * n2 * T(i, j, 2, 3, 3);
    case 81: return -l * (n2 - (l2 + m2) / 2) * T(j, i, 2, 3, 2) + S3 * l * n2 * T(j, i, 2, 3, 3);
    case 28: return m * (n2 - (l2 + m2) / 2) * T(i, j, 2, 3, 2) - S3 * m * n2 * T(i, j, 2, 3, 3);
    case 82: return -m * (n2 - (l2 + m2) / 2) * T(j, i, 2, 3, 2) + S3 * m * n2 * T(j, i, 2, 3, 3);
    case 38: return n * (n2 - (l2 + m2) / 2) * T(i, j, 2, 3, 2) + S3 * n * (l2 + m2) * T(i, j, 2, 3, 3);
    case 83: return -n * (n2 - (l2 + m2) / 2) * T(j, i, 2, 3, 2) - S3 * n * (l2 + m2) * T(j, i, 2, 3, 3);
    // d - d
    case 44:
      return 3 * l2 * m2 * T(i, j, 3, 3, 2) + (l2 + m2 - 4 * l2 * m2) * T(i, j, 3, 3, 3) +
             (n2 + l2 * m2) * T(i, j, 3, 3, 4);
    case 55:
      return 3 * m2 * n2 * T(i, j, 3, 3, 2) + (m2 + n2 - 4 * m2 * n2) * T(i, j, 3, 3, 3) +
             (l2 + m2 * n2) * T(i, j, 3, 3, 4);
    case 66:
      return 3 * l2 * n2 * T(i, j, 3, 3, 2) + (l2 + n2 - 4 * l2 * n2) * T(i, j, 3, 3, 3) +
             (m2 + l2 * n2) * T(i, j, 3, 3, 4);
    case 45:
      return 3 * l * m2 * n * T(i, j, 3, 3, 2) + l * n * (1 - 4 * m2) * T(i, j, 3, 3, 3) +
             l * n * (m2 - 1) * T(i, j, 3, 3, 4);
    case 54:
      return 3 * l * m2 * n * T(j, i, 3, 3, 2) + l * n * (1 - 4 * m2) * T(j, i, 3, 3, 3) +
             l * n * (m2 - 1) * T(j, i, 3, 3, 4);
    case 46:
      return 3 * m * l2 * n * T(i, j, 3, 3, 2) + m * n * (1 - 4 * l2) * T(i, j, 3, 3, 3) +
             m * n * (l2 - 1) * T(i, j, 3, 3, 4);
    case 64:
      return 3 * m * l2 * n * T(j, i, 3, 3, 2) + m * n * (1 - 4 * l2) * T(j, i, 3, 3, 3) +
             m * n * (l2 - 1) * T(j, i, 3, 3, 4);
    case 56:
      return 3 * m * n2 * l * T(i, j, 3, 3, 2) + m * l * (1 - 4 * n2) * T(i, j, 3, 3, 3) +
             m * l * (n2 - 1) * T(i, j, 3, 3, 4);
    case 65:
      return 3 * m * n2 * l * T(j, i, 3, 3, 2) + m * l * (1 - 4 * n2) * T(j, i, 3, 3, 3) +
             m * l * (n2 - 1) * T(j, i, 3, 3, 4);
    case 47:
      return (3.0 / 2) * l * m * (l2 - m2) * T(i, j, 3, 3, 2) + 2 * l * m * (m2 - l2) * T(i, j, 3, 3, 3) +
             (1.0 / 2) * l * m * (l2 - m2) * T(i, j, 3, 3, 4);
    case 74:
      return (3.0 / 2) * l * m * (l2 - m2) * T(j, i, 3, 3, 2) + 2 * l * m * (m2 - l2) * T(j, i, 3, 3, 3) +
             (1.0 / 2) * l * m * (l2 - m2) * T(j, i, 3, 3, 4);
    case 57:
      return (3.0 / 2) * m * n * (l2 - m2) * T(i, j, 3, 3, 2) - m * n * (1 + 2 * (l2 - m2)) * T(i, j, 3, 3, 3) +
             m * n * (1 + (l2 - m2) / 2) * T(i, j, 3, 3, 4);
    case 75:
      return (3.0 / 2) * m * n * (l2 - m2) * T(j, i, 3, 3, 2) - m * n * (1 + 2 * (l2 - m2)) * T(j, i, 3, 3, 3) +
             m * n * (1 + (l2 - m2) / 2) * T(j, i, 3, 3, 4);
    case 67:
      return (3.0 / 2) * l * n * (l2 - m2) * T(i, j, 3, 3, 2) + l * n * (1 - 2 * (l2 - m2)) * T(i, j, 3, 3, 3) -
             l * n * (1 - (l2 - m2) / 2) * T(i, j, 3, 3, 4);
    case 76:
      return (3.0 / 2) * l * n * (l2 - m2) * T(j, i, 3, 3, 2) + l * n * (1 - 2 * (l2 - m2)) * T(j, i, 3, 3, 3) -
             l * n * (1 - (l2 - m2) / 2) * T(j, i, 3, 3, 4);
    case 48:
      return S3 * l * m * (n2 - (l2 + m2) / 2) * T(i, j, 3, 3, 2) - (2 * S3) * l * m * n2 * T(i, j, 3, 3, 3) +
             (S3 / 2) * l * m * (1 + n2) * T(i, j, 3, 3, 4);
    case 84:
      return S3 * l * m * (n2 - (l2 + m2) / 2) * T(j, i, 3, 3, 2) - (2 * S3) * l * m * n2 * T(j, i, 3, 3, 3) +
             (S3 / 2) * l * m * (1 + n2) * T(j, i, 3, 3, 4);
    case 58:
      return S3 * m * n * (n2 - (l2 + m2) / 2) * T(i, j, 3, 3, 2) + S3 * m * n * (l2 + m2 - n2) * T(i, j, 3, 3, 3) -
             (S3 / 2) * m * n * (l2 + m2) * T(i, j, 3, 3, 4);
    case 85:
      return S3 * m * n * (n2 - (l2 + m2) / 2) * T(j, i, 3, 3, 2) + S3 * m * n * (l2 + m2 - n2) * T(j, i, 3, 3, 3) -
             (S3 / 2) * m * n * (l2 + m2) * T(j, i, 3, 3, 4);
    case 68:
      return S3 * l * n * (n2 - (l2 + m2) / 2) * T(i, j, 3, 3, 2) + S3 * l * n * (l2 + m2 - n2) * T(i, j, 3, 3, 3) -
             (S3 / 2) * l * n * (l2 + m2) * T(i, j, 3, 3, 4);
    case 86:
      return S3 * l * n * (n2 - (l2 + m2) / 2) * T(j, i, 3, 3, 2) + S3 * l * n * (l2 + m2 - n2) * T(j, i, 3, 3, 3) -
             (S3 / 2) * l * n * (l2 + m2) * T(j, i, 3, 3, 4);
    case 77:
      return (3.0 / 4) * ((l2 - m2) * (l2 - m2)) * T(i, j, 3, 3, 2) +
             (l2 + m2 - (l2 - m2) * (l2 - m2)) * T(i, j, 3, 3, 3) +
             (n2 + ((l2 - m2) * (l2 - m2)) / 4) * T(i, j, 3, 3, 4);
    case 78:
      return (S3 / 2) * (l2 - m2) * (n2 - (l2 + m2) / 2) * T(i, j, 3, 3, 2) + S3 * n2 * (m2 - l2) * T(i, j, 3, 3, 3) +
             (S3 / 4) * (1 + n2) * (l2 - m2) * T(i, j, 3, 3, 4);
    case 87:
      return (S3 / 2) * (l2 - m2) * (n2 - (l2 + m2) / 2) * T(j, i, 3, 3, 2) + S3 * n2 * (m2 - l2) * T(j, i, 3, 3, 3) +
             (S3 / 4) * (1 + n2) * (l2 - m2) * T(j, i, 3, 3, 4);
    case 88: {
      const double e = n2 - (l2 + m2) / 2;
      return (e * e) * T(j, i, 3, 3, 2) + 3 * n2 * (l2 + m2) * T(j, i, 3, 3, 3) +
             (3.0 / 4) * ((l2 + m2) * (l2 + m2)) * T(j, i, 3, 3, 4);
    }
    // s*
    case 99: return T(i, j, 4, 4, 2);
    case 9: return T(i, j, 1, 4, 2);
    case 90: return T(j, i, 1, 4, 2);
    case 91: return l * T(i, j, 4, 2, 2);
    case 19: return -l * T(j, i, 4, 2, 2);
    case 92: return m * T(i, j, 4, 2, 2);
    case 29: return -m * T(j, i, 4, 2, 2);
    case 93: return n * T(i, j, 4, 2, 2);
    case 39: return -n * T(j, i, 4, 2, 2);
    case 94: return S3 * (l * m) * T(i, j, 4, 3, 2);
    case 49: return S3 * (l * m) * T(j, i, 4, 3, 2);
    case 95: return S3 * (m * n) * T(i, j, 4, 3, 2);
    case 59: return S3 * (m * n) * T(j, i, 4, 3, 2);
    case 96: return S3 * (l * n) * T(i, j, 4, 3, 2);
    case 69: return S3 * (l * n) * T(j, i, 4, 3, 2);
    case 97: return (S3 / 2) * (l2 - m2) * T(i, j, 4, 3, 2);
    case 79: return (S3 / 2) * (l2 - m2) * T(j, i, 4, 3, 2);
    case 98: return (n2 - (l2 + m2) / 2) * T(i, j, 4, 3, 2);
    case 89: return (n2 - (l2 + m2) / 2) * T(j, i, 4, 3, 2);
    default: return 0.0;
  }
#undef T
}

// Raw gen_ham element between orbitals a and b (27 images, cutoff, phase).
__device__ double2 raw_elem(const TbArgs& A, int a, int b, double kx, double ky, double kz) {
  const int ia = A.oatom[a], ja = A.oatom[b];
  const int si = A.ospec[a], sj = A.ospec[b];
  const int oi = A.ocode[a], oj = A.ocode[b];
  double re = 0.0, im = 0.0;
  for (int i1 = -1; i1 <= 1; ++i1)
    for (int i2 = -1; i2 <= 1; ++i2)
      for (int i3 = -1; i3 <= 1; ++i3) {
        const double sx = i1 * A.lat[0] + i2 * A.lat[3] + i3 * A.lat[6];
        const double sy = i1 * A.lat[1] + i2 * A.lat[4] + i3 * A.lat[7];
        const double sz = i1 * A.lat[2] + i2 * A.lat[5] + i3 * A.lat[8];
        const double rx = A.pos[3 * ja] - A.pos[3 * ia] + sx;
        const double ry = A.pos[3 * ja + 1] - A.pos[3 * ia + 1] + sy;
        const double rz = A.pos[3 * ja + 2] - A.pos[3 * ia + 2] + sz;
        if (sqrt(rx * rx + ry * ry + rz * rz) < A.rcut) {
          const double v = (ia == ja) ? onsite(A, si, sj, oi, oj) : vsk(A, si, sj, oi, oj, rx, ry, rz);
          double s, c;
          sincos(rx * kx + ry * ky + rz * kz, &s, &c);
          re += c * v;
          im += s * v;
        }
      }
  return make_double2(re, im);
}

// Output element e of k point blockIdx.y: which block (diag / upper) and where.
__global__ void tb_kernel(TbArgs A, int nk, const double* kcart, int nblk, const int* blk_orb, const long long* eoff,
                          long long per_k, double* out) {
  const int k = blockIdx.y;
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= nk || e >= per_k) return;
  // block search: entries 0..nblk-1 diagonal, nblk..2nblk-2 upper couplings
  int lo = 0, hi = 2 * nblk - 2;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (eoff[mid] <= e) lo = mid; else hi = mid - 1;
  }
  const int blk = lo;
  const bool diag = blk < nblk;
  const int I = diag ? blk : blk - nblk;
  const int J = diag ? I : I + 1;
  const int rI = blk_orb[I], nI = blk_orb[I + 1] - blk_orb[I];
  const int cJ = blk_orb[J];
  const long long loc = e - eoff[blk];
  const int r = (int)(loc % nI), c = (int)(loc / nI);
  const int a = rI + r, b = cJ + c;
  const double kx = kcart[3 * k], ky = kcart[3 * k + 1], kz = kcart[3 * k + 2];
  const double2 hab = raw_elem(A, a, b, kx, ky, kz);
  const double2 hba = raw_elem(A, b, a, kx, ky, kz);
  // 0.5 (H + H^H)
  out[2 * ((size_t)k * per_k + e)] = 0.5 * (hab.x + hba.x);
  out[2 * ((size_t)k * per_k + e) + 1] = 0.5 * (hab.y - hba.y);
}

struct DevBuf {
  std::vector<void*> ptrs;
  ~DevBuf() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t up(T** d, const T* h, size_t n) {
    cudaError_t e = cudaMalloc((void**)d, n * sizeof(T) > 0 ? n * sizeof(T) : 1);
    if (e != cudaSuccess) return e;
    ptrs.push_back(*d);
    return n ? cudaMemcpy(*d, h, n * sizeof(T), cudaMemcpyHostToDevice) : cudaSuccess;
  }
};

}  // namespace

extern "C" {

const char* pf_tb_last_error(void) { return g_err; }

int pf_tb_hk_blocks(int natoms, const double* pos, const int* species, int nspecies, const int* norb_species,
                    const int* orb_codes, const double* V, const double* Vn, const double* r_d,
                    const double* latvec, const double* recivec, double r_cutoff, int nk, const double* kfrac,
                    int nblk, const int* blk_atom, double* out) {
  if (natoms <= 0 || nspecies <= 0 || nk <= 0 || nblk <= 0) return set_err(PF_ERR_ARG, "pf_tb: sizes must be positive");
  if (!pos || !species || !norb_species || !orb_codes || !V || !Vn || !r_d || !latvec || !recivec || !kfrac ||
      !blk_atom || !out)
    return set_err(PF_ERR_ARG, "pf_tb: null pointer");
  for (int s = 0; s < nspecies; ++s)
    if (norb_species[s] < 0 || norb_species[s] > PF_TB_MAX_ORB) return set_err(PF_ERR_ARG, "pf_tb: bad orbital count");
  // per-orbital tables in gen_ham's order (atom-major, species orbital list)
  std::vector<int> oatom, ospec, ocode, atom_first(natoms + 1, 0);
  for (int a = 0; a < natoms; ++a) {
    const int s = species[a];
    if (s < 0 || s >= nspecies) return set_err(PF_ERR_ARG, "pf_tb: species index out of range");
    atom_first[a] = (int)oatom.size();
    for (int o = 0; o < norb_species[s]; ++o) {
      const int code = orb_codes[s * PF_TB_MAX_ORB + o];
      if (code < 0 || code > 9) return set_err(PF_ERR_ARG, "pf_tb: orbital code must be 0..9");
      oatom.push_back(a);
      ospec.push_back(s);
      ocode.push_back(code);
    }
  }
  atom_first[natoms] = (int)oatom.size();
  std::vector<int> blk_orb(nblk + 1);
  for (int I = 0; I <= nblk; ++I) {
    if (blk_atom[I] < 0 || blk_atom[I] > natoms || (I > 0 && blk_atom[I] <= blk_atom[I - 1]))
      return set_err(PF_ERR_ARG, "pf_tb: block atom boundaries must increase within [0, natoms]");
    blk_orb[I] = atom_first[blk_atom[I]];
  }
  std::vector<long long> eoff(2 * nblk);
  long long e = 0;
  for (int I = 0; I < nblk; ++I) {
    eoff[I] = e;
    const long long nI = blk_orb[I + 1] - blk_orb[I];
    e += nI * nI;
  }
  for (int I = 0; I + 1 < nblk; ++I) {
    eoff[nblk + I] = e;
    e += (long long)(blk_orb[I + 1] - blk_orb[I]) * (blk_orb[I + 2] - blk_orb[I + 1]);
  }
  const long long per_k = e;
  std::vector<double> kc(3 * (size_t)nk);
  for (int k = 0; k < nk; ++k)
    for (int c = 0; c < 3; ++c)
      kc[3 * k + c] = kfrac[3 * k] * recivec[c] + kfrac[3 * k + 1] * recivec[3 + c] + kfrac[3 * k + 2] * recivec[6 + c];
  const size_t npair = (size_t)nspecies * nspecies;
  DevBuf d;
  TbArgs A;
  A.nspecies = nspecies;
  A.rcut = r_cutoff;
  for (int i = 0; i < 9; ++i) A.lat[i] = latvec[i];
  double *dV, *dVn, *drd, *dpos, *dk, *dout;
  int *doa, *dos, *doc, *dbo;
  long long* deo;
  cudaError_t err = cudaSuccess;
  if ((err = d.up(&dV, V, npair * 64)) != cudaSuccess || (err = d.up(&dVn, Vn, npair * 64)) != cudaSuccess ||
      (err = d.up(&drd, r_d, npair)) != cudaSuccess || (err = d.up(&dpos, pos, 3 * (size_t)natoms)) != cudaSuccess ||
      (err = d.up(&doa, oatom.data(), oatom.size())) != cudaSuccess ||
      (err = d.up(&dos, ospec.data(), ospec.size())) != cudaSuccess ||
      (err = d.up(&doc, ocode.data(), ocode.size())) != cudaSuccess ||
      (err = d.up(&dbo, blk_orb.data(), blk_orb.size())) != cudaSuccess ||
      (err = d.up(&deo, eoff.data(), eoff.size())) != cudaSuccess ||
      (err = d.up(&dk, kc.data(), kc.size())) != cudaSuccess) {
    snprintf(g_err, sizeof(g_err), "pf_tb: %s", cudaGetErrorString(err));
    return PF_ERR_CUDA;
  }
  const size_t outn = 2 * (size_t)nk * per_k;
  if ((err = cudaMalloc((void**)&dout, outn * 8)) != cudaSuccess) {
    snprintf(g_err, sizeof(g_err), "pf_tb: %s", cudaGetErrorString(err));
    return PF_ERR_CUDA;
  }
  d.ptrs.push_back(dout);
  A.V = dV;
  A.Vn = dVn;
  A.r_d = drd;
  A.pos = dpos;
  A.oatom = doa;
  A.ospec = dos;
  A.ocode = doc;
  const dim3 grid((unsigned)((per_k + 127) / 128), (unsigned)nk);
  tb_kernel<<<grid, 128>>>(A, nk, dk, nblk, dbo, deo, per_k, dout);
  if ((err = cudaGetLastError()) == cudaSuccess) err = cudaMemcpy(out, dout, outn * 8, cudaMemcpyDeviceToHost);
  if (err != cudaSuccess) {
    snprintf(g_err, sizeof(g_err), "pf_tb: %s", cudaGetErrorString(err));
    return PF_ERR_CUDA;
  }
  return PF_SUCCESS;
}

}  // extern "C"
