// Binary force-constant (full-Hamiltonian) path of the phonon code:
//   * gen_dyn      (negf/dyn.f90:39-150)   dense norb x norb D(q), THz^2, Hermitised
//   * gen_dyn_lead (negf/dyn.f90:190-312)  lead layer D(q) (Hermitised) and its
//                                           coupling to the next layer (not Hermitised)
// both from the reduced index tables of gen_fc_to_dyn_idx /
// gen_lead_fc_to_dyn_idx (negf/dyn.f90:988-1216, flattened row-major over the
// atom pairs as negf/phinfortran.f90:655-683 does), and
//   * the slices negf/surface.f90:170-198 and negf/device.f90:323-500 take from
//     the dense matrix, written as the block set of the tdb transport entries
//     (every device layer zero-padded to a common size n).
// One thread per (k, atom pair, cartesian pair) accumulates the pair's
// entries in the reference's order; a second kernel forms 0.5 (H + H^H).
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
int cuda_err(cudaError_t e) {
  snprintf(g_err, sizeof(g_err), "pf_fullh: %s", cudaGetErrorString(e));
  return PF_ERR_CUDA;
}

constexpr double kEleVolt = 1.609e-19;         // negf/util.f90:7
constexpr double kMassProton = 1.6726219e-27;  // negf/util.f90:8
constexpr double kPi = 3.141592653589793238;   // negf/util.f90:5

struct FcPairs {
  int npairs;
  const int* pa;        // pair row atom
  const int* pb;        // pair column atom
  const int* off;       // [npairs + 1] entry offsets
  const int* eidx;      // fc column atom of every entry (0-based)
  const double* edr;    // [nent][3] bond vectors
  const int* row_atom;  // [natoms] fc row atom (0-based, central cell)
  const double* mass;   // [natoms]
  const double* fc;     // column-major fc_rows x fc_cols
  int fc_rows;
};

// H[q] (column-major, norb x norb) += the 3x3 block of every pair; the
// untouched elements were zeroed by the caller.
__global__ void gen_dyn_kernel(FcPairs P, int norb, int nq, const double* kc, double2* H) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long total = (long long)nq * P.npairs * 9;
  if (t >= total) return;
  const int e9 = (int)(t % 9);
  const long long pq = t / 9;
  const int pr = (int)(pq % P.npairs);
  const int q = (int)(pq / P.npairs);
  const int ic = e9 / 3, jc = e9 % 3;
  const int a = P.pa[pr], b = P.pb[pr];
  const double s = sqrt(P.mass[a] * P.mass[b]);
  const double k0 = kc[3 * q], k1 = kc[3 * q + 1], k2 = kc[3 * q + 2];
  const size_t row = 3 * (size_t)P.row_atom[a] + ic;
  double re = 0.0, im = 0.0;
  for (int e = P.off[pr]; e < P.off[pr + 1]; ++e) {
    const double* d = P.edr + 3 * (size_t)e;
    const double x = d[0] * k0 + d[1] * k1 + d[2] * k2;
    double sn, cs;
    sincos(x, &sn, &cs);
    const double f = P.fc[row + (3 * (size_t)P.eidx[e] + jc) * (size_t)P.fc_rows];
    re += f * cs / s;   // (fc * exp(i dr.k)) / sqrt(m1 m2)
    im += f * sn / s;
  }
  // THz^2: Ham*eleVolt/1.0d-20/mass_proton/(1.0d12*2.0d0*pi)**2, left to right
  const double w = 1.0e12 * 2.0 * kPi;
  const double w2 = w * w;
  re = re * kEleVolt / 1.0e-20 / kMassProton / w2;
  im = im * kEleVolt / 1.0e-20 / kMassProton / w2;
  H[(size_t)q * norb * norb + (3 * (size_t)b + jc) * norb + 3 * (size_t)a + ic] = make_double2(re, im);
}

// H <- 0.5 (H + H^H) per k (negf/util.f90:940-949); thread (r, c) with r <= c
// writes both elements.
__global__ void hermitize_kernel(int norb, int nq, double2* H) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long per = (long long)norb * norb;
  if (t >= per * nq) return;
  const int q = (int)(t / per);
  const long long rc = t % per;
  const int r = (int)(rc % norb), c = (int)(rc / norb);
  if (r > c) return;
  double2* M = H + (size_t)q * per;
  const double2 x = M[r + (size_t)c * norb], y = M[c + (size_t)r * norb];
  M[r + (size_t)c * norb] = make_double2(0.5 * (x.x + y.x), 0.5 * (x.y - y.y));
  if (r != c) M[c + (size_t)r * norb] = make_double2(0.5 * (y.x + x.x), 0.5 * (y.y - x.y));
}

struct TdbOut {
  double2 *HL, *HLv, *HR, *HRv, *Hd, *Hdv, *Hld, *Hrd;
};

// Every block element of every k: the block families in ABI order, each
// [k][block][col][row].  Device layer j spans rows/columns
// d0 + ls[j] .. d0 + ls[j+1] - 1 of the dense matrix; entries past the
// layer's own size are the zero padding.
__global__ void dense_to_tdb_kernel(int norb, int nq, const double2* H, int nl, int nr, int nbl, int nbr, int L,
                                    int n, const int* ls, TdbOut o, int* bad) {
  const long long cnt[8] = {(long long)nl * nl, (long long)nl * nl, (long long)nr * nr, (long long)nr * nr,
                            (long long)L * n * n, (long long)(L > 1 ? L - 1 : 0) * n * n, (long long)nl * n,
                            (long long)nr * n};
  long long per = 0;
  for (int f = 0; f < 8; ++f) per += cnt[f];
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= per * nq) return;
  const int q = (int)(t / per);
  long long e = t % per;
  int f = 0;
  while (e >= cnt[f]) e -= cnt[f++];
  const int d0 = nbl + 2 * nl, ol = nbl + nl, il = nbl, orr = norb - nbr - 2 * nr, ir = norb - nbr - nr;
  int rows, blk = 0, r, c, gr = -1, gc = -1;
  bool inside = true;
  switch (f) {
    case 0: case 1: rows = nl; break;
    case 2: case 3: rows = nr; break;
    case 6: rows = nl; break;
    case 7: rows = nr; break;
    default: rows = n; blk = (int)(e / ((long long)n * n)); e %= (long long)n * n; break;
  }
  r = (int)(e % rows);
  c = (int)(e / rows);
  switch (f) {
    case 0: gr = ol + r; gc = ol + c; break;
    case 1: gr = il + r; gc = ol + c; break;
    case 2: gr = orr + r; gc = orr + c; break;
    case 3: gr = ir + r; gc = orr + c; break;
    case 4: {
      const int dj = ls[blk + 1] - ls[blk];
      inside = r < dj && c < dj;
      gr = d0 + ls[blk] + r;
      gc = d0 + ls[blk] + c;
      break;
    }
    case 5: {
      const int dj = ls[blk + 1] - ls[blk], dk = ls[blk + 2] - ls[blk + 1];
      inside = r < dj && c < dk;
      gr = d0 + ls[blk] + r;
      gc = d0 + ls[blk + 1] + c;
      break;
    }
    case 6: inside = c < ls[1] - ls[0]; gr = ol + r; gc = d0 + ls[0] + c; break;
    default: inside = c < ls[L] - ls[L - 1]; gr = orr + r; gc = d0 + ls[L - 1] + c; break;
  }
  double2 v = make_double2(0.0, 0.0);
  if (inside) {
    if (gr < 0 || gr >= norb || gc < 0 || gc >= norb) {
      atomicOr(bad, 1);
    } else {
      v = H[(size_t)q * norb * norb + (size_t)gc * norb + gr];
    }
  }
  double2* dst[8] = {o.HL, o.HLv, o.HR, o.HRv, o.Hd, o.Hdv, o.Hld, o.Hrd};
  const long long base = (long long)q * cnt[f];
  const long long inblk = (f == 4 || f == 5) ? (long long)blk * n * n + r + (long long)c * n : r + (long long)c * rows;
  dst[f][base + inblk] = v;
}

int launch_gen_dyn(const FcPairs& P, int norb, int nq, const double* kc, int hermitize, double* H, cudaStream_t st) {
  const size_t bytes = (size_t)nq * norb * norb * sizeof(double2);
  cudaError_t e = cudaMemsetAsync(H, 0, bytes, st);
  if (e != cudaSuccess) return cuda_err(e);
  const long long total = (long long)nq * P.npairs * 9;
  if (total > 0) {
    gen_dyn_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(P, norb, nq, kc, reinterpret_cast<double2*>(H));
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e);
  }
  if (hermitize) {
    const long long tt = (long long)nq * norb * norb;
    hermitize_kernel<<<(unsigned)((tt + 255) / 256), 256, 0, st>>>(norb, nq, reinterpret_cast<double2*>(H));
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_err(e);
  }
  return PF_SUCCESS;
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

const char* pf_fullh_last_error(void) { return g_err; }

int pf_gen_dyn_dev(int natoms, int fc_rows, const double* fc, int npairs, const int* pair_a, const int* pair_b,
                   const int* pair_off, const int* ent_idx, const double* ent_dr, const int* row_atom,
                   const double* mass, int nq, const double* kcart, int hermitize, double* H, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (natoms <= 0 || fc_rows <= 0 || npairs < 0 || nq <= 0) return set_err(PF_ERR_ARG, "pf_gen_dyn: bad sizes");
  if (!fc || !row_atom || !mass || !kcart || !H || (npairs > 0 && (!pair_a || !pair_b || !pair_off || !ent_idx ||
                                                                    !ent_dr)))
    return set_err(PF_ERR_ARG, "pf_gen_dyn: null pointer");
  FcPairs P{npairs, pair_a, pair_b, pair_off, ent_idx, ent_dr, row_atom, mass, fc, fc_rows};
  return launch_gen_dyn(P, 3 * natoms, nq, kcart, hermitize, H, stream);
}

int pf_gen_dyn(int natoms, int nbx, int nby, int n_uc, int nz, int fc_rows, int fc_cols, const double* fc,
               const int* num_mat, int nent, const int* idx_mat_red, const double* dist_mat_red, const double* mass,
               const double* recivec, int nq, const double* kpoints, int hermitize, double* Ham) {
  if (natoms <= 0 || nbx <= 0 || nby <= 0 || n_uc <= 0 || nz <= 0 || nq <= 0 || nent < 0)
    return set_err(PF_ERR_ARG, "pf_gen_dyn: sizes must be positive");
  if (n_uc % nz != 0 || natoms != nbx * nby * n_uc)
    return set_err(PF_ERR_ARG, "pf_gen_dyn: natoms must be nbx*nby*n_uc and n_uc a multiple of nz");
  if (fc_rows != 3 * n_uc || fc_cols <= 0 || fc_cols % 3 != 0)
    return set_err(PF_ERR_ARG, "pf_gen_dyn: force-constant rows must be 3*n_uc, columns a multiple of 3");
  if (!fc || !num_mat || !mass || !recivec || !kpoints || !Ham || (nent > 0 && (!idx_mat_red || !dist_mat_red)))
    return set_err(PF_ERR_ARG, "pf_gen_dyn: null pointer");
  // pairs in the reference's (a, b) row-major walk; num_mat is Fortran
  // column-major (num_mat(a+1, b+1) at a + b*natoms)
  std::vector<int> pa, pb, off(1, 0), row(natoms), eidx(nent);
  std::vector<double> edr(3 * (size_t)nent);
  long long seen = 0;
  for (int a = 0; a < natoms; ++a) {
    for (int b = 0; b < natoms; ++b) {
      const int c = num_mat[a + (size_t)b * natoms];
      if (c < 0) return set_err(PF_ERR_ARG, "pf_gen_dyn: negative num_mat entry");
      if (c == 0) continue;
      seen += c;
      if (seen > nent) return set_err(PF_ERR_ARG, "pf_gen_dyn: num_mat sums past the entry list");
      pa.push_back(a);
      pb.push_back(b);
      off.push_back((int)seen);
    }
  }
  if (seen != nent) return set_err(PF_ERR_ARG, "pf_gen_dyn: num_mat does not sum to the entry count");
  for (int e = 0; e < nent; ++e) {
    const int j = idx_mat_red[e];
    if (j < 1 || 3 * (long long)j > fc_cols) return set_err(PF_ERR_ARG, "pf_gen_dyn: fc column atom out of range");
    eidx[e] = j - 1;
    for (int c = 0; c < 3; ++c) edr[3 * (size_t)e + c] = dist_mat_red[e + (size_t)c * nent];
  }
  // fc row atom of every atom (negf/dyn.f90:95-103; nz = 1 is gen_dyn_lead's rule)
  const int per = n_uc / nz;
  for (int a = 0; a < natoms; ++a) {
    const int iz = a / (nby * nbx * per);
    int rem = a - iz * nby * nbx * per;
    const int iy = rem / (nbx * per);
    rem -= iy * nbx * per;
    const int ix = rem / per;
    row[a] = iz * per + (rem - ix * per);
  }
  std::vector<double> kc(3 * (size_t)nq);
  for (int q = 0; q < nq; ++q)
    for (int c = 0; c < 3; ++c)
      kc[3 * q + c] = kpoints[3 * q] * recivec[c] + kpoints[3 * q + 1] * recivec[3 + c] +
                      kpoints[3 * q + 2] * recivec[6 + c];
  DevBuf d;
  double *dfc, *dedr, *dmass, *dkc, *dH;
  int *dpa, *dpb, *doff, *deidx, *drow;
  cudaError_t err;
  const int np = (int)pa.size();
  if ((err = d.up(&dfc, fc, (size_t)fc_rows * fc_cols)) != cudaSuccess ||
      (err = d.up(&dedr, edr.data(), edr.size())) != cudaSuccess ||
      (err = d.up(&dmass, mass, (size_t)natoms)) != cudaSuccess ||
      (err = d.up(&dkc, kc.data(), kc.size())) != cudaSuccess ||
      (err = d.up(&dpa, pa.data(), pa.size())) != cudaSuccess ||
      (err = d.up(&dpb, pb.data(), pb.size())) != cudaSuccess ||
      (err = d.up(&doff, off.data(), off.size())) != cudaSuccess ||
      (err = d.up(&deidx, eidx.data(), eidx.size())) != cudaSuccess ||
      (err = d.up(&drow, row.data(), row.size())) != cudaSuccess)
    return cuda_err(err);
  const int norb = 3 * natoms;
  const size_t hbytes = (size_t)nq * norb * norb * sizeof(double2);
  if ((err = cudaMalloc((void**)&dH, hbytes)) != cudaSuccess) return cuda_err(err);
  d.ptrs.push_back(dH);
  FcPairs P{np, dpa, dpb, doff, deidx, dedr, drow, dmass, dfc, fc_rows};
  const int rc = launch_gen_dyn(P, norb, nq, dkc, hermitize, dH, 0);
  if (rc != PF_SUCCESS) return rc;
  if ((err = cudaMemcpy(Ham, dH, hbytes, cudaMemcpyDeviceToHost)) != cudaSuccess) return cuda_err(err);
  return PF_SUCCESS;
}

int pf_dense_to_tdb_dev(int norb, int nq, const double* H, int nl, int nr, int n_buffer_l, int n_buffer_r, int L,
                        const int* layer_start, int n, double* HL, double* HLv, double* HR, double* HRv, double* Hd,
                        double* Hdv, double* Hld, double* Hrd, int* bad, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (norb <= 0 || nq <= 0 || nl <= 0 || nr <= 0 || n_buffer_l < 0 || n_buffer_r < 0 || L <= 0 || n <= 0)
    return set_err(PF_ERR_ARG, "pf_dense_to_tdb: bad sizes");
  if (n_buffer_l + 2 * nl + n_buffer_r + 2 * nr >= norb)
    return set_err(PF_ERR_ARG, "pf_dense_to_tdb: no device orbitals left between the lead cells");
  if (!H || !layer_start || !HL || !HLv || !HR || !HRv || !Hd || (L > 1 && !Hdv) || !Hld || !Hrd || !bad)
    return set_err(PF_ERR_ARG, "pf_dense_to_tdb: null pointer");
  const long long per = 2LL * nl * nl + 2LL * nr * nr + (long long)L * n * n + (long long)(L - 1) * n * n +
                        (long long)nl * n + (long long)nr * n;
  const long long total = per * nq;
  TdbOut o{reinterpret_cast<double2*>(HL), reinterpret_cast<double2*>(HLv), reinterpret_cast<double2*>(HR),
           reinterpret_cast<double2*>(HRv), reinterpret_cast<double2*>(Hd), reinterpret_cast<double2*>(Hdv),
           reinterpret_cast<double2*>(Hld), reinterpret_cast<double2*>(Hrd)};
  dense_to_tdb_kernel<<<(unsigned)((total + 255) / 256), 256, 0, stream>>>(
      norb, nq, reinterpret_cast<const double2*>(H), nl, nr, n_buffer_l, n_buffer_r, L, n, layer_start, o, bad);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PF_SUCCESS : cuda_err(e);
}

}  // extern "C"
