// Block dynamical-matrix assembly D(q) of the tdb branch on the GPU.
//
// Reference: gen_dyn_qe_tdb_k (negf/dyn.f90:1482-2080).  For one transverse
// q the reference fills eight block families (Haml, Hamlv, Hamr, Hamrv,
// Hamd(L), Hamdv(L-1), Hamld, Hamrd); element (3bi+m, 3bj+n) of a block is
//   sum_{a,b} w(dr) fc(m,n,idx_i,idx_j,t1,t2,t3) exp(i dr.k) / sqrt(m_i m_j),
//   dr = -(a,b,0).cell_all + pos_j - pos_i,
//   w(dr) = 1/nreq from the 124 Wigner-Seitz planes (dyn.f90:1571-1586),
//   (t1,t2,t3) from the lattice offset of dr (dyn.f90:1587-1606).
// Everything but the phase is independent of q, so the GPU splits it:
//   1. term_kernel: one thread per (block, atom pair, image) evaluates the
//      WS weight, the IFC cell index and dr once (a q-independent table);
//   2. phase_kernel: one thread per (q, block, atom pair, m, n) sums the
//      images in the reference's loop order (a outer, b inner).
// Inputs use the reference's Fortran layouts (column-major arrays,
// 1-based idxall) so the driver passes its own arrays.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "../../include/phinfortran_gb300.h"

namespace {

thread_local char g_err[512] = "";

int set_err(int code, const char* msg) {
  snprintf(g_err, sizeof(g_err), "%s", msg);
  return code;
}
int cuda_err(cudaError_t e, const char* where) {
  snprintf(g_err, sizeof(g_err), "%s: %s", where, cudaGetErrorString(e));
  return PF_ERR_CUDA;
}
#define DY_CUDA(call)                                  \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_err(e_, #call); \
  } while (0)

// One block family: atom ranges (0-based, contiguous) for rows and columns,
// number of blocks (layers) and the output offset of its first block.
struct Family {
  int row0, col0;     // first atom of block 0
  int row_step, col_step;  // atom offset between consecutive blocks (layers)
  int nrow, ncol;     // atoms per block
  int nblk;           // blocks in the family
  size_t out_off;     // complex offset of block 0 in the family's q-stacked output
  size_t q_stride;    // complex elements per q of the family
};

struct Geometry {
  int nat, nx, ny, nz, natall, nscx, nscy, nab;
  const double* fc;        // fc(3,3,nat,nat,nx,ny,nz)
  const double* pos;       // pos(nat,3)
  const double* pos_all;   // pos_all(natall,3)
  const int* idxall;       // 1-based
  const double* mass_all;  // (natall)
  const double* rws;       // rws(124,3)
  const double* rd;        // (124)
  double cell_all[9];      // cell_all(3,3), row i = vector i
  double ivcell[9];        // inv(cell) (ivcell(3,3) as in dyn.f90:1540)
};

// Term table entry for one (block, atom pair, image).
struct Term {
  double coef;   // w / sqrt(m_i m_j) (0: no contribution)
  double dr[3];
  int fc_off;    // offset of fc(1,1,idx_i,idx_j,t1,t2,t3)
};

__device__ __forceinline__ double rnd_away(double x) { return x >= 0 ? floor(x + 0.5) : -floor(-x + 0.5); }

__global__ void term_kernel(Geometry g, const Family* fam, int nfam, const size_t* pair_base, Term* terms,
                            size_t total) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    // locate family
    int f = 0;
    while (f + 1 < nfam && pair_base[f + 1] * g.nab <= t) ++f;
    const Family F = fam[f];
    const size_t local = t - pair_base[f] * g.nab;
    const int ab = (int)(local % g.nab);
    const size_t pr = local / g.nab;          // pair index within family: ((blk*nrow + bi)*ncol + bj)
    const int bj = (int)(pr % F.ncol);
    const int bi = (int)((pr / F.ncol) % F.nrow);
    const int blk = (int)(pr / ((size_t)F.ncol * F.nrow));
    const int i = F.row0 + blk * F.row_step + bi;
    const int j = F.col0 + blk * F.col_step + bj;
    const int a = ab / (2 * g.nscy + 1) - g.nscx;
    const int b = ab % (2 * g.nscy + 1) - g.nscy;
    const int ii = g.idxall[i] - 1, jj = g.idxall[j] - 1;
    double dr[3], du[3];
    for (int d = 0; d < 3; ++d) {
      const double shift = a * g.cell_all[0 + 3 * d] + b * g.cell_all[1 + 3 * d];
      dr[d] = -shift + g.pos_all[j + (size_t)g.natall * d] - g.pos_all[i + (size_t)g.natall * d];
      du[d] = dr[d] - (g.pos[jj + g.nat * d] - g.pos[ii + g.nat * d]);
    }
    // ixyz = du . ivcell   (row vector times matrix, dyn.f90:1570)
    double ixyz[3];
    for (int c = 0; c < 3; ++c) ixyz[c] = du[0] * g.ivcell[0 + 3 * c] + du[1] * g.ivcell[1 + 3 * c] + du[2] * g.ivcell[2 + 3 * c];
    int nreq = 1;
    bool outside = false;
    for (int ir = 0; ir < 124; ++ir) {
      const double df = dr[0] * g.rws[ir] + dr[1] * g.rws[ir + 124] + dr[2] * g.rws[ir + 248] - g.rd[ir];
      if (df > 1.0e-5) {
        outside = true;
        continue;
      }
      if (fabs(df) <= 1.0e-5) ++nreq;
    }
    Term T;
    T.coef = 0.0;
    T.fc_off = 0;
    T.dr[0] = dr[0];
    T.dr[1] = dr[1];
    T.dr[2] = dr[2];
    if (!outside) {
      const int aa = -(int)rnd_away(ixyz[0]), bb = -(int)rnd_away(ixyz[1]), cc = -(int)rnd_away(ixyz[2]);
      int t1 = ((aa % g.nx) + g.nx) % g.nx, t2 = ((bb % g.ny) + g.ny) % g.ny, t3 = ((cc % g.nz) + g.nz) % g.nz;
      T.coef = (1.0 / nreq) / sqrt(g.mass_all[i] * g.mass_all[j]);
      T.fc_off = 9 * (ii + g.nat * (jj + g.nat * (t1 + g.nx * (t2 + g.ny * t3))));
    }
    terms[t] = T;
  }
}

// One thread per (q, family pair, m, n): sum over images in (a, b) order.
__global__ void phase_kernel(Geometry g, const Family* fam, int nfam, const size_t* pair_base, const Term* terms,
                             const double* kpt /*(nq,3) cartesian*/, int nq, size_t npairs,
                             double2* const* outs) {
  const size_t total = (size_t)nq * npairs * 9;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const int mn = (int)(t % 9);
    const size_t rest = t / 9;
    const size_t gp = rest % npairs;           // global pair index
    const int q = (int)(rest / npairs);
    int f = 0;
    while (f + 1 < nfam && pair_base[f + 1] <= gp) ++f;
    const Family F = fam[f];
    const size_t pr = gp - pair_base[f];
    const int bj = (int)(pr % F.ncol);
    const int bi = (int)((pr / F.ncol) % F.nrow);
    const int blk = (int)(pr / ((size_t)F.ncol * F.nrow));
    const int m = mn % 3, n = mn / 3;
    const double k0 = kpt[q], k1 = kpt[q + nq], k2 = kpt[q + 2 * nq];
    double re = 0.0, im = 0.0;
    const Term* tt = terms + gp * g.nab;
    for (int ab = 0; ab < g.nab; ++ab) {
      const Term T = tt[ab];
      if (T.coef > 0.0) {
        const double v = T.coef * g.fc[T.fc_off + m + 3 * n];
        double s, c;
        sincos(T.dr[0] * k0 + T.dr[1] * k1 + T.dr[2] * k2, &s, &c);
        re += v * c;
        im += v * s;
      }
    }
    const int rows = 3 * F.nrow;
    const size_t el = F.out_off + (size_t)q * F.q_stride + (size_t)blk * rows * (3 * F.ncol) +
                      (size_t)(3 * bi + m) + (size_t)rows * (3 * bj + n);
    outs[f][el] = make_double2(re, im);
  }
}

void inv3(const double* a, double* r) {
  // a, r in Fortran (3,3) layout: a(i,j) = a[i + 3j]
  const double det = a[0] * (a[4] * a[8] - a[7] * a[5]) - a[3] * (a[1] * a[8] - a[7] * a[2]) +
                     a[6] * (a[1] * a[5] - a[4] * a[2]);
  r[0] = (a[4] * a[8] - a[7] * a[5]) / det;
  r[3] = -(a[3] * a[8] - a[6] * a[5]) / det;
  r[6] = (a[3] * a[7] - a[6] * a[4]) / det;
  r[1] = -(a[1] * a[8] - a[7] * a[2]) / det;
  r[4] = (a[0] * a[8] - a[6] * a[2]) / det;
  r[7] = -(a[0] * a[7] - a[6] * a[1]) / det;
  r[2] = (a[1] * a[5] - a[4] * a[2]) / det;
  r[5] = -(a[0] * a[5] - a[3] * a[2]) / det;
  r[8] = (a[0] * a[4] - a[3] * a[1]) / det;
}

}  // namespace

extern "C" {

const char* pf_dyn_last_error(void) { return g_err; }

int pf_gen_dyn_qe_tdb(int nat, int nx, int ny, int nz, const double* fc, const double* cell, const double* cell_all,
                      const double* pos, int natall, const double* pos_all, const int* idxall,
                      const double* mass_all, const double* rws, const double* rd, int n_bloch_x, int n_bloch_y,
                      int buffer_left, int period_left, int buffer_right, int period_right, int nlayer,
                      int natm_layer, int nq, const double* kgrid, double* HL, double* HLv, double* HR,
                      double* HRv, double* Hd, double* Hdv, double* Hld, double* Hrd) {
  if (nat <= 0 || nx <= 0 || ny <= 0 || nz <= 0 || natall <= 0 || n_bloch_x <= 0 || n_bloch_y <= 0 || nlayer <= 0 ||
      natm_layer <= 0 || nq <= 0 || period_left <= 0 || period_right <= 0)
    return set_err(PF_ERR_ARG, "pf_gen_dyn_qe_tdb: dimensions must be positive");
  if (!fc || !cell || !cell_all || !pos || !pos_all || !idxall || !mass_all || !rws || !rd || !kgrid || !HL || !HLv ||
      !HR || !HRv || !Hd || !Hld || !Hrd || (nlayer > 1 && !Hdv))
    return set_err(PF_ERR_ARG, "pf_gen_dyn_qe_tdb: null pointer");
  const int bl = buffer_left, pl = period_left, br = buffer_right, pr = period_right, N = natall;
  const int ds = bl + 2 * pl;
  if (ds + nlayer * natm_layer > N - br - 2 * pr || bl < 0 || br < 0)
    return set_err(PF_ERR_ARG, "pf_gen_dyn_qe_tdb: atom ranges exceed the structure");
  for (int i = 0; i < N; ++i)
    if (idxall[i] < 1 || idxall[i] > nat) return set_err(PF_ERR_ARG, "pf_gen_dyn_qe_tdb: idxall out of range");
  Geometry g;
  g.nat = nat;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.natall = N;
  g.nscx = (nx + n_bloch_x - 1) / n_bloch_x;   // ceiling(nx/nx_sc), dyn.f90:1545
  g.nscy = (ny + n_bloch_y - 1) / n_bloch_y;
  g.nab = (2 * g.nscx + 1) * (2 * g.nscy + 1);
  // Fortran cell(3,3) -> row-vector convention: element (i,d) at [i + 3d]
  for (int k = 0; k < 9; ++k) g.cell_all[k] = cell_all[k];
  inv3(cell, g.ivcell);
  // kpoint = kgrid . cell_reci, cell_reci = 2 pi inv(cell)^T  (dyn.f90:1547-1560)
  const double two_pi = 2.0 * 3.141592653589793238;
  std::vector<double> kc((size_t)nq * 3);
  for (int q = 0; q < nq; ++q)
    for (int c = 0; c < 3; ++c) {
      double s = 0.0;
      for (int r = 0; r < 3; ++r) s += kgrid[q + (size_t)nq * r] * two_pi * g.ivcell[c + 3 * r];
      kc[q + (size_t)nq * c] = s;
    }
  const int na = natm_layer;
  const size_t nl3 = 3 * pl, nr3 = 3 * pr, n3 = 3 * na;
  // families in the reference order
  Family fam[8] = {
      {bl, bl, 0, 0, pl, pl, 1, 0, nl3 * nl3},                                          // Haml
      {bl, bl + pl, 0, 0, pl, pl, 1, 0, nl3 * nl3},                                     // Hamlv
      {N - br - pr, N - br - pr, 0, 0, pr, pr, 1, 0, nr3 * nr3},                        // Hamr
      {N - br - pr, N - br - 2 * pr, 0, 0, pr, pr, 1, 0, nr3 * nr3},                    // Hamrv
      {ds, ds, na, na, na, na, nlayer, 0, (size_t)nlayer * n3 * n3},                    // Hamd
      {ds, ds + na, na, na, na, na, nlayer - 1, 0, (size_t)(nlayer - 1) * n3 * n3},     // Hamdv
      {bl + pl, ds, 0, 0, pl, na, 1, 0, nl3 * n3},                                      // Hamld
      {N - br - 2 * pr, ds + (nlayer - 1) * na, 0, 0, pr, na, 1, 0, nr3 * n3}};         // Hamrd
  double* hostout[8] = {HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd};
  std::vector<Family> fv;
  std::vector<double*> hv;
  std::vector<size_t> base;
  size_t npairs = 0;
  for (int f = 0; f < 8; ++f) {
    if (fam[f].nblk <= 0) continue;
    base.push_back(npairs);
    npairs += (size_t)fam[f].nblk * fam[f].nrow * fam[f].ncol;
    fv.push_back(fam[f]);
    hv.push_back(hostout[f]);
  }
  const int nfam = (int)fv.size();
  base.push_back(npairs);
  const size_t fc_n = (size_t)9 * nat * nat * nx * ny * nz;
  // device buffers
  double *d_fc = nullptr, *d_pos = nullptr, *d_posall = nullptr, *d_mass = nullptr, *d_rws = nullptr,
         *d_rd = nullptr, *d_k = nullptr;
  int* d_idx = nullptr;
  Family* d_fam = nullptr;
  size_t* d_base = nullptr;
  Term* d_terms = nullptr;
  double2** d_outs = nullptr;
  std::vector<double2*> d_o(nfam, nullptr);
  int rc = PF_SUCCESS;
  auto cleanup = [&]() {
    cudaFree(d_fc);
    cudaFree(d_pos);
    cudaFree(d_posall);
    cudaFree(d_mass);
    cudaFree(d_rws);
    cudaFree(d_rd);
    cudaFree(d_k);
    cudaFree(d_idx);
    cudaFree(d_fam);
    cudaFree(d_base);
    cudaFree(d_terms);
    cudaFree(d_outs);
    for (auto p : d_o) cudaFree(p);
  };
#define DY_TRY(call)                  \
  do {                                \
    cudaError_t e_ = (call);          \
    if (e_ != cudaSuccess) {          \
      rc = cuda_err(e_, #call);       \
      cleanup();                      \
      return rc;                      \
    }                                 \
  } while (0)
  DY_TRY(cudaMalloc(&d_fc, fc_n * 8));
  DY_TRY(cudaMalloc(&d_pos, (size_t)nat * 3 * 8));
  DY_TRY(cudaMalloc(&d_posall, (size_t)N * 3 * 8));
  DY_TRY(cudaMalloc(&d_mass, (size_t)N * 8));
  DY_TRY(cudaMalloc(&d_rws, 124 * 3 * 8));
  DY_TRY(cudaMalloc(&d_rd, 124 * 8));
  DY_TRY(cudaMalloc(&d_k, (size_t)nq * 3 * 8));
  DY_TRY(cudaMalloc(&d_idx, (size_t)N * 4));
  DY_TRY(cudaMalloc(&d_fam, nfam * sizeof(Family)));
  DY_TRY(cudaMalloc(&d_base, (nfam + 1) * sizeof(size_t)));
  DY_TRY(cudaMalloc(&d_terms, npairs * g.nab * sizeof(Term)));
  DY_TRY(cudaMalloc(&d_outs, nfam * sizeof(double2*)));
  for (int f = 0; f < nfam; ++f) DY_TRY(cudaMalloc(&d_o[f], (size_t)nq * fv[f].q_stride * 16));
  DY_TRY(cudaMemcpy(d_fc, fc, fc_n * 8, cudaMemcpyHostToDevice));
  DY_TRY(cudaMemcpy(d_pos, pos, (size_t)nat * 3 * 8, cudaMemcpyHostToDevice));
  DY_TRY(cudaMemcpy(d_posall, pos_all, (size_t)N * 3 * 8, cudaMemcpyHostToDevice));
  DY_TRY(cudaMemcpy(d_mass, mass_all, (size_t)N * 8, cudaMemcpyHostToDevice));
  DY_TRY(cudaMemcpy(d_rws, rws, 124 * 3 * 8, cudaMemcpyHostToDevice));
  DY_TRY(cudaMemcpy(d_rd, rd, 124 * 8, cudaMemcpyHostToDevice));
  DY_TRY(cudaMemcpy(d_k, kc.data(), (size_t)nq * 3 * 8, cudaMemcpyHostToDevice));
  DY_TRY(cudaMemcpy(d_idx, idxall, (size_t)N * 4, cudaMemcpyHostToDevice));
  DY_TRY(cudaMemcpy(d_fam, fv.data(), nfam * sizeof(Family), cudaMemcpyHostToDevice));
  DY_TRY(cudaMemcpy(d_base, base.data(), (nfam + 1) * sizeof(size_t), cudaMemcpyHostToDevice));
  DY_TRY(cudaMemcpy(d_outs, d_o.data(), nfam * sizeof(double2*), cudaMemcpyHostToDevice));
  g.fc = d_fc;
  g.pos = d_pos;
  g.pos_all = d_posall;
  g.idxall = d_idx;
  g.mass_all = d_mass;
  g.rws = d_rws;
  g.rd = d_rd;
  const size_t tt = npairs * g.nab;
  term_kernel<<<(int)((tt + 255) / 256 < 65535 ? (tt + 255) / 256 : 65535), 256>>>(g, d_fam, nfam, d_base, d_terms,
                                                                                   tt);
  DY_TRY(cudaGetLastError());
  const size_t pt = (size_t)nq * npairs * 9;
  phase_kernel<<<(int)((pt + 255) / 256 < 65535 ? (pt + 255) / 256 : 65535), 256>>>(g, d_fam, nfam, d_base, d_terms,
                                                                                    d_k, nq, npairs, d_outs);
  DY_TRY(cudaGetLastError());
  for (int f = 0; f < nfam; ++f)
    DY_TRY(cudaMemcpy(hv[f], d_o[f], (size_t)nq * fv[f].q_stride * 16, cudaMemcpyDeviceToHost));
  cleanup();
  return PF_SUCCESS;
#undef DY_TRY
}

}  // extern "C"
