/*
 * phinfortran_gb300.h -- C ABI of the GB300 NEGF transport engine.
 *
 * Drop-in for the per-(ie,ik) hot loop of KitchenSong/phinfortran's tdb
 * transport branch (negf/phinfortran.f90:1188-1251).  The Fortran driver
 * keeps its input readers, grids and output writers and calls these
 * functions through iso_c_binding.
 *
 * Conventions (those of the reference's arrays):
 *  - every matrix is complex(kind=8), column-major, passed as double* to
 *    interleaved (re, im) pairs; element (r, c) of an m-row block sits at
 *    [2*(r + c*m)] / [2*(r + c*m) + 1];
 *  - per-q block sets are stacked: HL[q][nl*nl], Hd[q][L][n*n], ...;
 *  - "tdb" block names follow negf/dyn.f90:1482-2080:
 *      HL  = Haml   left lead cell onsite        (nl x nl)
 *      HLv = Hamlv  H_{-1,0}  lead cell coupling (nl x nl)
 *      HR  = Hamr   right lead cell onsite       (nr x nr)
 *      HRv = Hamrv  H_{N+2,N+1}                  (nr x nr)
 *      Hd  = Hamd   device layer onsite          (L blocks, n x n)
 *      Hdv = Hamdv  H_{i,i+1}                    (L-1 blocks, n x n)
 *      Hld = Hamld  H_{0,1}                      (nl x n)
 *      Hrd = Hamrd  H_{N+1,N}                    (nr x n)
 *  - energies are the reference's Egrid values (omega^2 in THz^2 for the
 *    phonon driver, E for the electron driver);
 *  - lead broadening eps = E*eta + eta0 (negf/surface.f90:479); the device
 *    uses E + i*dev_factor*eps (dev_factor = 10 reproduces
 *    negf/lesser.f90:556, 1 reproduces tb/device.f90:390 with eta = 0,
 *    eta0 = the tb eta);
 *  - transmissions below 1e-60 are returned as 0 (negf/lesser.f90:795-800)
 *    and points flagged in zero_flag return 0 (the ie == 1 rule,
 *    negf/lesser.f90:802-807).
 *
 * Return codes: PF_SUCCESS, a negative PF_ERR_* for argument / CUDA
 * errors, or PF_ERR_POINT when any point's status word is nonzero (the
 * reference would `stop` there: util.f90:29-66).  pf_last_error() gives a
 * message.  Per-point status bits: 1 singular block, 2 non-finite value,
 * 4 decimation reached max_iter (the reference loop is unbounded,
 * negf/surface.f90:488).
 */
#ifndef PHINFORTRAN_GB300_H
#define PHINFORTRAN_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PF_ABI_VERSION 1

#define PF_SUCCESS 0
#define PF_ERR_ARG (-1)
#define PF_ERR_CUDA (-2)
#define PF_ERR_SIZE (-3)
#define PF_ERR_POINT (-4)

/* Largest block dimension (n, nl, nr) of the shared-memory resident kernel. */
#define PF_NMAX_RESIDENT 48

/* Message for the last error on the calling thread. */
const char* pf_last_error(void);

/* ABI version (PF_ABI_VERSION of the built library). */
int pf_version(void);

/*
 * Fused transport for a batch of (omega, q) points, device pointers.
 *
 * Replaces, per point p = (ie, ik):
 *   surface_green_tdb_mpi(ie, ik, ...)   negf/surface.f90:344-383
 *     (left advanced and right retarded decimations, Sigma, Gamma)
 *   get_G_full_tdb_mpi(ie, ik, ...)      negf/lesser.f90:100-157
 *     (left-to-right sweep, right lead closure, Caroli transl;
 *      with want_transr also the right-to-left sweep and transr)
 * i.e. the transmission part of negf/phinfortran.f90:1196-1213 and, with
 * dev_factor = 1, of tb/infortran.f90:490-501 (surface_green + G_block).
 *
 * E[npts], qidx[npts] (may be NULL: all q = 0), zero_flag[npts] (may be
 * NULL) and the outputs transl[npts], transr[npts], status[npts],
 * iters[2*npts] (left, right iteration counts; may be NULL) are device
 * arrays.  work must hold pf_transport_tdb_workspace_size(n, nl, nr, nq,
 * npts) bytes of device memory.  When the right lead blocks equal the left
 * ones bitwise (HR == HL, HRv == HLv for a q), the right retarded surface
 * function is taken as the adjoint of the left advanced one instead of a
 * second decimation (exact identity for hermitian leads).  stream is a cudaStream_t (NULL: default stream).
 * The call is asynchronous on `stream`.
 */
size_t pf_transport_tdb_workspace_size(int n, int nl, int nr, int nq, int npts);

int pf_transport_tdb_dev(int n, int nl, int nr, int L, int nq,
                         const double* HL, const double* HLv,
                         const double* HR, const double* HRv,
                         const double* Hd, const double* Hdv,
                         const double* Hld, const double* Hrd,
                         int npts, const double* E, const int* qidx,
                         const int* zero_flag,
                         double eta, double eta0, double dev_factor,
                         double convergence, int max_iter, int want_transr,
                         double* transl, double* transr, int* status,
                         int* iters, void* work, size_t work_bytes,
                         void* stream);

/*
 * Same computation with HOST pointers for every array (what the Fortran
 * driver holds).  Copies in, runs on the current device, copies out and
 * synchronises.  Device buffers are cached between calls.
 */
int pf_transport_tdb(int n, int nl, int nr, int L, int nq,
                     const double* HL, const double* HLv,
                     const double* HR, const double* HRv,
                     const double* Hd, const double* Hdv,
                     const double* Hld, const double* Hrd,
                     int npts, const double* E, const int* qidx,
                     const int* zero_flag,
                     double eta, double eta0, double dev_factor,
                     double convergence, int max_iter, int want_transr,
                     double* transl, double* transr, int* status,
                     int* iters);

/*
 * Mixed-precision transport (T_L only), device pointers.  Same inputs and
 * meaning as pf_transport_tdb_dev; the arithmetic differs:
 *   - the lead decimations (negf/surface.f90:488-497) for blocks up to 32
 *     run in FP64 arithmetic with their block products on the tensor cores
 *     (exact BF16 slice products): the doubling iteration amplifies its
 *     own rounding, and near subband edges at eta ~ 1e-6 double-float
 *     (48-bit) decimations leave T up to 5e-8 away from FP64 even where
 *     FP64 itself is reproducible.  Above 32 they run in double-float
 *     (pairs of FP32 numbers on the FP32 pipe): there FP64 decimations have
 *     no tensor-core path and cost twice the whole double-float solve
 *     (PF_ARITH_AUTO; pf_transport_tdb_mixed_ex_dev chooses explicitly);
 *   - the device blocks are factorised in FP32 (the left-connected
 *     recursion of negf/lesser.f90:547-654 as a block LU of the extended
 *     lead+device matrix), and the last block column G_{:,N+1} is refined
 *     against a double-float residual: one sweep for every point, then up
 *     to refine_iters - 1 more for each point whose last correction of the
 *     block X_0 = G_{0,N+1} was above 3e-5 (PF_REFINE_TOL) relative to X_0 (refine_iters
 *     in [0, 16]; 0 keeps the FP32 solution);
 *   - the Caroli trace (negf/lesser.f90:787-792) is taken in double-float.
 * work must hold pf_transport_tdb_mixed_workspace_size(...) bytes.
 */
size_t pf_transport_tdb_mixed_workspace_size(int n, int nl, int nr, int L,
                                             int nq, int npts);

int pf_transport_tdb_mixed_dev(int n, int nl, int nr, int L, int nq,
                               const double* HL, const double* HLv,
                               const double* HR, const double* HRv,
                               const double* Hd, const double* Hdv,
                               const double* Hld, const double* Hrd,
                               int npts, const double* E, const int* qidx,
                               const int* zero_flag,
                               double eta, double eta0, double dev_factor,
                               double convergence, int max_iter,
                               int refine_iters, double* transl, int* status,
                               int* iters, void* work, size_t work_bytes,
                               void* stream);

/*
 * pf_transport_tdb_mixed_dev with the lead arithmetic chosen by lead_arith:
 * PF_ARITH_AUTO (what pf_transport_tdb_mixed_dev does: PF_ARITH_FP64 for
 * blocks up to 32, PF_ARITH_DF64 above), PF_ARITH_FP64 (whole decimations
 * in FP64; block products on the tensor cores up to 32, FP64 SIMT above),
 * PF_ARITH_SPLIT (the first 8 decimation steps in FP64, the rest in
 * double-float) or PF_ARITH_DF64 (whole decimations in double-float).  Same
 * workspace size.
 */
#define PF_ARITH_SPLIT 3
#define PF_ARITH_AUTO (-1)
int pf_transport_tdb_mixed_ex_dev(int n, int nl, int nr, int L, int nq,
                                  const double* HL, const double* HLv,
                                  const double* HR, const double* HRv,
                                  const double* Hd, const double* Hdv,
                                  const double* Hld, const double* Hrd,
                                  int npts, const double* E, const int* qidx,
                                  const int* zero_flag,
                                  double eta, double eta0, double dev_factor,
                                  double convergence, int max_iter,
                                  int refine_iters, int lead_arith,
                                  double* transl, int* status, int* iters,
                                  void* work, size_t work_bytes, void* stream);

/* Host-pointer variant of pf_transport_tdb_mixed_dev (synchronous). */
int pf_transport_tdb_mixed(int n, int nl, int nr, int L, int nq,
                           const double* HL, const double* HLv,
                           const double* HR, const double* HRv,
                           const double* Hd, const double* Hdv,
                           const double* Hld, const double* Hrd,
                           int npts, const double* E, const int* qidx,
                           const int* zero_flag,
                           double eta, double eta0, double dev_factor,
                           double convergence, int max_iter, int refine_iters,
                           double* transl, int* status, int* iters);

/*
 * Block dynamical matrices of the tdb branch for nq transverse q points,
 * assembled on the GPU.  Replaces gen_dyn_qe_tdb_k (negf/dyn.f90:1482-2080),
 * called by gen_dyn_qe_tdb_mpi once per k (negf/phinfortran.f90:1189).
 * Inputs are the reference's own arrays, Fortran layout:
 *   fc(3,3,nat,nat,nx,ny,nz) (THz^2 amu, after cutoff and ASR, fc.f90:204-266),
 *   cell(3,3) (QE cell, row i = vector i), cell_all(3,3) (supercell),
 *   pos(nat,3), pos_all(natall,3), idxall(natall) (1-based basis index),
 *   mass_all(natall), rws(124,3), rd(124) (fc.f90:271-289),
 *   kgrid(nq,3) fractional (config.f90:153-188 after k_grid_in_ws).
 * Outputs (host arrays, interleaved complex, the layout pf_transport_tdb
 * takes): HL,HLv [nq][3pl x 3pl], HR,HRv [nq][3pr x 3pr],
 * Hd [nq][nlayer][3na x 3na], Hdv [nq][nlayer-1][3na x 3na],
 * Hld [nq][3pl x 3na], Hrd [nq][3pr x 3na]  (pl = period_left,
 * pr = period_right, na = natm_layer).  Like the reference, the blocks are
 * not hermitised.
 */
int pf_gen_dyn_qe_tdb(int nat, int nx, int ny, int nz, const double* fc,
                      const double* cell, const double* cell_all,
                      const double* pos, int natall, const double* pos_all,
                      const int* idxall, const double* mass_all,
                      const double* rws, const double* rd,
                      int n_bloch_x, int n_bloch_y,
                      int buffer_left, int period_left,
                      int buffer_right, int period_right,
                      int nlayer, int natm_layer,
                      int nq, const double* kgrid,
                      double* HL, double* HLv, double* HR, double* HRv,
                      double* Hd, double* Hdv, double* Hld, double* Hrd);

/* Message for the last error of pf_gen_dyn_qe_tdb on the calling thread. */
const char* pf_dyn_last_error(void);

/*
 * Two-probe Landauer conductance for ntemp temperatures (host arrays):
 * sigma[t] = 1/area * 1/(2 pi) * trapz(hbar w df/dT trans(w), w), the
 * formula of examples/negf/si-si/condt.py:14-30 (omega in rad/s, SI units,
 * trans already averaged over k as condt.py:44-51 does).
 */
int pf_landauer_conductance(int ne, const double* omega, const double* trans,
                            int ntemp, const double* temps, double area,
                            double* sigma);

/* Message for the last error of pf_landauer_conductance. */
const char* pf_cond_last_error(void);

/*
 * Adjoint of the transmission (FP64), device pointers.  No counterpart in
 * the reference (the derivative that an inverse design or a thermal-
 * conductance optimisation needs).  For the points of a batch with weights
 * w_p (NULL: all 1; points with zero_flag get weight 0) it returns T_L of
 * every point (as pf_transport_tdb_dev) and accumulates
 *     M_B = sum_p w_p dT_p/dB,   dF = Re Tr[dB M_B],  F = sum_p w_p T_p,
 * for the device blocks and the lead-device couplings:
 *   gHd [nq][L][n x n], gHdv [nq][L-1][n x n], gHld [nq][n x nl],
 *   gHrd [nq][n x nr]  (device arrays, interleaved complex, zeroed here).
 * The lead cells (HL, HLv, HR, HRv) are held fixed.
 * ckpt: checkpoint interval of the left-connected factors.  0 picks
 * ceil(sqrt(L + 2)): the factors and forward vectors are kept every ckpt
 * layers and each segment is recomputed during the reverse pass (memory
 * O(sqrt(L)) matrices per point in flight); 1 keeps every layer (memory
 * O(L), no recomputation, less work).
 * arith: PF_ARITH_FP64 (complex128 throughout) or PF_ARITH_DF64 (every
 * block operation in double-float pairs on the FP32 pipe, ~48 significant
 * bits; the blocks are converted once into the workspace).
 * work must hold pf_transport_tdb_grad_workspace_size(...) bytes.
 */
#define PF_ARITH_FP64 0
#define PF_ARITH_DF64 1
/* The FP64 algorithm with its block products on the tensor cores as exact
 * BF16 slice products (see pf_tc_zgemm_dev); large-block entry only. */
#define PF_ARITH_TC 2

size_t pf_transport_tdb_grad_workspace_size(int n, int nl, int nr, int L,
                                            int nq, int npts, int ckpt,
                                            int arith);

int pf_transport_tdb_grad_dev(int n, int nl, int nr, int L, int nq,
                              const double* HL, const double* HLv,
                              const double* HR, const double* HRv,
                              const double* Hd, const double* Hdv,
                              const double* Hld, const double* Hrd,
                              int npts, const double* E, const int* qidx,
                              const int* zero_flag, const double* weights,
                              double eta, double eta0, double dev_factor,
                              double convergence, int max_iter, int ckpt,
                              int arith,
                              double* transl, int* status, int* iters,
                              double* gHd, double* gHdv, double* gHld,
                              double* gHrd, void* work, size_t work_bytes,
                              void* stream);

/* Message for the last error of the gradient entry points. */
const char* pf_grad_last_error(void);

/*
 * Allocation-free variant of pf_transport_tdb_dev.  No counterpart in the
 * reference (whose Fortran arrays are all allocated by the driver): it
 * serves callers that cannot give this library a device workspace -- host
 * codes that reserve the GPU's memory up front through their own allocator
 * and forbid any later cudaMalloc.  It takes the same device arrays as
 * pf_transport_tdb_dev minus `work`/`work_bytes` and calls no cudaMalloc,
 * cudaFree or allocating library routine.  Its scratch is a static device
 * array of PF_NOALLOC_SCRATCH_BYTES that every GPU loading the library
 * holds until the process exits; problems whose minimum scratch exceeds it
 * are rejected with PF_ERR_SIZE, and large batches run with fewer
 * concurrent CTAs.  The first call on a device resolves the array's device
 * address (cudaGetSymbolAddress, with that device current); make that first
 * call before any stream capture.  The address belongs to the device's
 * CUDA context: after a device reset the next call resolves it again, so
 * that call too must come before any capture.  All calls share the array: calls whose
 * kernels overlap on the GPU (concurrent streams, several host threads)
 * race on it and must be serialised by the caller.
 */
#define PF_NOALLOC_SCRATCH_BYTES (32u << 20)

int pf_transport_tdb_noalloc(int n, int nl, int nr, int L, int nq,
                             const double* HL, const double* HLv,
                             const double* HR, const double* HRv,
                             const double* Hd, const double* Hdv,
                             const double* Hld, const double* Hrd,
                             int npts, const double* E, const int* qidx,
                             const int* zero_flag,
                             double eta, double eta0, double dev_factor,
                             double convergence, int max_iter, int want_transr,
                             double* transl, double* transr, int* status,
                             int* iters, void* stream);

/*
 * Mode-resolved transmission (replaces vel_mat_tdb_mpi,
 * negf/velocity_mat.f90:227-279, with vel_mat_tdb at
 * negf/velocity_mat.f90:1692-3148, called per (ie, ik) from
 * negf/phinfortran.f90:1238-1250 together with the surface and RGF calls
 * that feed it).  FP64.  For each point it runs the four lead
 * decimations, both sweeps and the Caroli traces (transl/transr as
 * pf_transport_tdb_dev with want_transr = 1), then the Bloch eigenmodes of
 * the four transfer matrices, the velocity matrices, the t/r matrices and
 * their specular / non-specular sums, written to mode_sums[8*p + k] in the
 * order transl_s, transl_ns, transr_s, transr_ns, refll_s, refll_ns,
 * reflr_s, reflr_ns (the reduce arrays of the reference's driver).
 *   lambda_eta        : propagating test | |lambda| - 1 | < lambda_eta
 *   a_z_l, a_z_r      : lead periods along transport (a_z_L, a_z_R)
 *   nshift            : folded k shifts (n_bloch_x * n_bloch_y)
 *   stride_*, nrep_*  : orbital stride between transverse images of the
 *                       lead layer and the orbitals of one image
 *   phase_l, phase_r  : unfolding phases [nq][nshift][nl|nr] complex,
 *                       exp(-i(-p.k_sc + (p - p_uc).k_shift)) per orbital
 *                       (velocity_mat.f90:2035-2072); built by the caller
 *   nprop             : optional [npts][4] propagating-mode counts of the
 *                       adv-L, ret-L, ret-R, adv-R problems
 * Points flagged in zero_flag get zero t/r sums (the ie == 1 rule).
 * Status bit 8: a Schur (QR) iteration did not converge.
 */
size_t pf_transport_tdb_modes_workspace_size(int n, int nl, int nr, int nq, int npts);

int pf_transport_tdb_modes_dev(int n, int nl, int nr, int L, int nq,
                               const double* HL, const double* HLv,
                               const double* HR, const double* HRv,
                               const double* Hd, const double* Hdv,
                               const double* Hld, const double* Hrd,
                               int npts, const double* E, const int* qidx,
                               const int* zero_flag,
                               double eta, double eta0, double dev_factor,
                               double convergence, int max_iter,
                               double lambda_eta, double a_z_l, double a_z_r,
                               int nshift, int stride_l, int nrep_l,
                               const double* phase_l, int stride_r, int nrep_r,
                               const double* phase_r,
                               double* transl, double* transr,
                               double* mode_sums, int* status, int* nprop,
                               void* work, size_t work_bytes, void* stream);

/*
 * pf_transport_tdb_modes_dev plus the per-mode data of the reference's
 * per-k mode files (write_specular / write_md, negf/write_data.f90:3-176,
 * called from negf/velocity_mat.f90:3108-3128), with mm = max(nl, nr) and
 * the four problems in the order adv-L, ret-L, ret-R, adv-R:
 *   mode_kz  [npts][4][mm]  k_z of every Bloch mode (k_z_L_ret etc.,
 *                           velocity_mat.f90:2360), 100 when the mode is
 *                           not propagating; modes in the order of this
 *                           library's eigen-solver
 *   mode_bz  [npts][4][mm]  unfolding label (bz_idx_*, 1-based; 0 when not
 *                           propagating)
 *   col_sums [npts][4][mm][nshift]  for the matrices tlr, trl, rrr, rll
 *                           (rows: the outgoing modes, columns: the
 *                           incoming ones) the sum of |M_rc|^2 over the
 *                           rows r of each label, per labelled column c
 * The in-plane k of a label is move_in_ws2((k_sc + shift) . recivec) and
 * depends on the label only, so the specular test of write_specular
 * (|k_f - k_b|^2 < 1e-5 in plane) is decided per label on the host.  All
 * three pointers are given or all are null.
 */
int pf_transport_tdb_modes_permode_dev(int n, int nl, int nr, int L, int nq,
                                       const double* HL, const double* HLv,
                                       const double* HR, const double* HRv,
                                       const double* Hd, const double* Hdv,
                                       const double* Hld, const double* Hrd,
                                       int npts, const double* E,
                                       const int* qidx, const int* zero_flag,
                                       double eta, double eta0,
                                       double dev_factor, double convergence,
                                       int max_iter, double lambda_eta,
                                       double a_z_l, double a_z_r, int nshift,
                                       int stride_l, int nrep_l,
                                       const double* phase_l, int stride_r,
                                       int nrep_r, const double* phase_r,
                                       double* transl, double* transr,
                                       double* mode_sums, int* status,
                                       int* nprop, double* mode_kz,
                                       int* mode_bz, double* col_sums,
                                       void* work, size_t work_bytes,
                                       void* stream);

/*
 * pf_transport_tdb_modes_permode_dev with flags (the three per-mode outputs
 * may all be null).  PF_MODES_ELECTRON selects the electron normalisation of
 * tb/velocity_mat.f90 (vel_mat, :222-1560): velocity matrices U^H Gamma U
 * (:467) and t / r = i V^1/2 U^-1 G U^-H V^1/2 (:1352-1370) with none of
 * the phonon factors a_z / (2 sqrt(E)) and 2 sqrt(E / (a_z a_z)); those
 * cancel in t and r for E > 0, and only the electron form is defined for
 * E <= 0 (energies below the band centre).  lambda_eta is the caller's
 * (the tb driver uses 1e-3, tb/velocity_mat.f90:355).
 */
#define PF_MODES_ELECTRON 1

int pf_transport_tdb_modes_ex_dev(int n, int nl, int nr, int L, int nq,
                                  const double* HL, const double* HLv,
                                  const double* HR, const double* HRv,
                                  const double* Hd, const double* Hdv,
                                  const double* Hld, const double* Hrd,
                                  int npts, const double* E,
                                  const int* qidx, const int* zero_flag,
                                  double eta, double eta0,
                                  double dev_factor, double convergence,
                                  int max_iter, double lambda_eta,
                                  double a_z_l, double a_z_r, int nshift,
                                  int stride_l, int nrep_l,
                                  const double* phase_l, int stride_r,
                                  int nrep_r, const double* phase_r, int flags,
                                  double* transl, double* transr,
                                  double* mode_sums, int* status,
                                  int* nprop, double* mode_kz,
                                  int* mode_bz, double* col_sums,
                                  void* work, size_t work_bytes,
                                  void* stream);

/*
 * pf_transport_tdb_modes_ex_dev plus the whole mode-to-mode matrices of
 * vel_mat_tdb, what write_md2md prints with verbosity = 1
 * (negf/velocity_mat.f90:3132-3145, negf/write_data.f90:177-241):
 * md2md[npts][4][mm][mm] (mm = max(nl, nr); matrices tlr, trl, rrr, rll;
 * column c, row r at [p][matrix][c][r]) = |M_rc|^2, rows the outgoing modes
 * of mode_kz's problem (ret-L, ret-R, ret-R, ret-L), columns the incoming
 * (adv-R, adv-L, adv-R, adv-L), zero outside the lead sizes and at points
 * with zero_flag.  md2md needs the per-mode outputs; null md2md is
 * pf_transport_tdb_modes_ex_dev.
 */
int pf_transport_tdb_modes_md2md_dev(int n, int nl, int nr, int L, int nq,
                                     const double* HL, const double* HLv,
                                     const double* HR, const double* HRv,
                                     const double* Hd, const double* Hdv,
                                     const double* Hld, const double* Hrd,
                                     int npts, const double* E,
                                     const int* qidx, const int* zero_flag,
                                     double eta, double eta0,
                                     double dev_factor, double convergence,
                                     int max_iter, double lambda_eta,
                                     double a_z_l, double a_z_r, int nshift,
                                     int stride_l, int nrep_l,
                                     const double* phase_l, int stride_r,
                                     int nrep_r, const double* phase_r, int flags,
                                     double* transl, double* transr,
                                     double* mode_sums, int* status,
                                     int* nprop, double* mode_kz,
                                     int* mode_bz, double* col_sums,
                                     double* md2md,
                                     void* work, size_t work_bytes,
                                     void* stream);

/*
 * The FP64 transport of one batch (T_L, T_R, status) plus the Green's
 * functions that the reference's vel_mat_tdb receives from
 * surface_green_tdb_mpi (negf/surface.f90:344-383: the four decimations)
 * and get_G_full_tdb_mpi (negf/lesser.f90:100-157), for drivers that keep
 * their own mode analysis.  Per point, column-major complex(kind=8), each
 * output optional (null: not written):
 *   gl_adv, gl_plus    [npts][nl][nl]  left surface functions (advanced,
 *                                      and the "plus" problem of :510-532)
 *   gr_ret, gr_minus   [npts][nr][nr]  right (retarded, "minus" :571-593)
 *   gml_adv [npts][nl][nl], gmr_ret [npts][nr][nr]   broadenings
 *                                      i (Sigma - Sigma^H)
 *   G_D_LR  [npts][nl][nr]  G_{0,N+1}     G_R [npts][nr][nr]  G_{N+1,N+1}
 *   G_D_RL  [npts][nr][nl]  G_{N+1,0}     G_L [npts][nl][nl]  G_{0,0}
 * The workspace is that of the mode-resolved entry
 * (pf_transport_tdb_blocks_workspace_size); errors are reported through
 * pf_modes_last_error.
 */
size_t pf_transport_tdb_blocks_workspace_size(int n, int nl, int nr, int nq, int npts);

int pf_transport_tdb_blocks_dev(int n, int nl, int nr, int L, int nq,
                                const double* HL, const double* HLv,
                                const double* HR, const double* HRv,
                                const double* Hd, const double* Hdv,
                                const double* Hld, const double* Hrd,
                                int npts, const double* E, const int* qidx,
                                const int* zero_flag, double eta, double eta0,
                                double dev_factor, double convergence,
                                int max_iter, double* transl, double* transr,
                                int* status, double* gl_adv, double* gl_plus,
                                double* gr_ret, double* gr_minus,
                                double* gml_adv, double* gmr_ret,
                                double* G_D_LR, double* G_R, double* G_D_RL,
                                double* G_L, void* work, size_t work_bytes,
                                void* stream);

/*
 * Stage timing of the mixed pipeline (blocks up to 32).  No reference
 * counterpart (profiling aid).  After pf_mixed_stage_timing(1) every mixed
 * call records CUDA events on its stream; pf_mixed_stage_times(ms, n >= 3)
 * waits for the last call's events and writes the durations in ms of
 * (0) the block conversions and sparse copies, (1) the lead decimations
 * (one kernel), (2) the factorisation, refinement and Caroli sweeps, and
 * returns 3 (or a negative error code; message in pf_last_error).  Off by
 * default; timed calls must not overlap and must not be captured into a
 * CUDA graph.
 */
int pf_mixed_stage_timing(int on);
int pf_mixed_stage_times(float* ms, int n);

/* Message for the last error of the mode-resolved entry points. */
const char* pf_modes_last_error(void);

/*
 * Large-block transport (FP64): the same quantities as
 * pf_transport_tdb_dev with want_transr = 0 (T_L, status, iterations) for
 * block sizes above PF_NMAX_RESIDENT, up to PF_NMAX_TILED.  Replaces the
 * same reference calls as pf_transport_tdb_dev (surface_green_tdb_mpi,
 * negf/surface.f90:344-383, and get_G_full_tdb_mpi, negf/lesser.f90:100-157)
 * for cross-sections whose blocks do not fit in shared memory.  Points are
 * grouped by q and advanced in batches through batched tile kernels (block
 * GEMMs, a blocked Gauss-Jordan inverse, masked decimation steps).  The call
 * is synchronous with respect to `stream` (the decimation loop reads one
 * counter per step).  arith: PF_ARITH_FP64, PF_ARITH_DF64 (every block
 * operation in double-float pairs on the FP32 pipe, ~48 significant bits;
 * the q block set is converted once into the workspace) or PF_ARITH_TC (the
 * FP64 algorithm with every block product on the tcgen05 tensor cores as
 * exact BF16 slice products, FP64-grade; the inverse panels stay FP64).
 * work: pf_transport_tdb_tiled_workspace_size bytes.
 */
#define PF_NMAX_TILED 2048

size_t pf_transport_tdb_tiled_workspace_size(int n, int nl, int nr, int L, int nq,
                                             int npts, int arith);

int pf_transport_tdb_tiled_dev(int n, int nl, int nr, int L, int nq,
                               const double* HL, const double* HLv,
                               const double* HR, const double* HRv,
                               const double* Hd, const double* Hdv,
                               const double* Hld, const double* Hrd,
                               int npts, const double* E, const int* qidx,
                               const int* zero_flag,
                               double eta, double eta0, double dev_factor,
                               double convergence, int max_iter, int arith,
                               double* transl, int* status, int* iters,
                               void* work, size_t work_bytes, void* stream);

/* pf_transport_tdb_tiled_dev with circular_flag = 1: the lead surface
 * Green's functions through circular_g (negf/circular.f90:42-105, called
 * from surface_green_tdb, negf/surface.f90:498-501 and :558-562) instead of
 * the decimation of the full lead matrices.  The leads are block circulant
 * over n_bloch_y x n_bloch_x Bloch cells (nl == nr, a multiple of
 * n_bloch_y * n_bloch_x): the first block rows of H00 and of the coupling are
 * Fourier-transformed along y (n_bloch_y outer blocks) and then x
 * (n_bloch_x inner blocks) (util.f90:732-756), the K = n_bloch_y * n_bloch_x
 * small blocks of nl / K are decimated on their own with beta = alpha^H
 * (util.f90:761-799), and the result is transformed back with the unitary
 * matrices of set_pmatrix (circular.f90:9-38).  gr (host, 4 doubles): the
 * G.R products of the forward transforms, {left y, left x, right y, right x}
 * = {reci_uc_l(2,:).latvec_uc_l(2,:), reci_uc_l(1,:).latvec_uc_l(1,:), the
 * same of the right lead}; the back transform takes the left lead's two, as
 * the reference builds P1, P2 once from the left lead
 * (negf/phinfortran.f90:622-628).  iters reports, per lead, the most
 * decimation steps of the K small blocks.  Only the first block rows of the
 * lead matrices are read, as in the reference, so leads that are not block
 * circulant give the reference's (wrong) result, not an error.  work:
 * pf_transport_tdb_tiled_circ_workspace_size bytes (0: invalid arguments). */
size_t pf_transport_tdb_tiled_circ_workspace_size(int n, int nl, int nr, int L, int nq,
                                                  int npts, int arith, int n_bloch_y,
                                                  int n_bloch_x);

int pf_transport_tdb_tiled_circ_dev(int n, int nl, int nr, int L, int nq,
                                    const double* HL, const double* HLv,
                                    const double* HR, const double* HRv,
                                    const double* Hd, const double* Hdv,
                                    const double* Hld, const double* Hrd,
                                    int npts, const double* E, const int* qidx,
                                    const int* zero_flag,
                                    double eta, double eta0, double dev_factor,
                                    double convergence, int max_iter, int arith,
                                    int n_bloch_y, int n_bloch_x, const double* gr,
                                    double* transl, int* status, int* iters,
                                    void* work, size_t work_bytes, void* stream);

/* The large-block entry with every option: the block-circulant leads of
 * pf_transport_tdb_tiled_circ_dev (n_bloch_y = n_bloch_x = 1: off, gr may
 * be NULL, any nl, nr) and, when transr is not NULL, T_R as well: the
 * right-to-left sweep of get_G_full_tdb (negf/lesser.f90:694-784) with the
 * left closure G_{0,0} = inv(z - H_L - Sigma_L - H_ld g_1 H_ld^H) and
 * T_R = Re Tr[G_{N+1,0} Gamma_L G_{N+1,0}^H Gamma_R] (:794-800), a second
 * sweep's cost.  work: pf_transport_tdb_tiled_ex_workspace_size bytes. */
size_t pf_transport_tdb_tiled_ex_workspace_size(int n, int nl, int nr, int L, int nq,
                                                int npts, int arith, int n_bloch_y,
                                                int n_bloch_x);

int pf_transport_tdb_tiled_ex_dev(int n, int nl, int nr, int L, int nq,
                                  const double* HL, const double* HLv,
                                  const double* HR, const double* HRv,
                                  const double* Hd, const double* Hdv,
                                  const double* Hld, const double* Hrd,
                                  int npts, const double* E, const int* qidx,
                                  const int* zero_flag,
                                  double eta, double eta0, double dev_factor,
                                  double convergence, int max_iter, int arith,
                                  int n_bloch_y, int n_bloch_x, const double* gr,
                                  double* transl, double* transr, int* status,
                                  int* iters, void* work, size_t work_bytes,
                                  void* stream);

/* Message for the last error of the large-block entry points. */
const char* pf_tiled_last_error(void);

/*
 * Tuning of the large-block path (no reference counterpart; set by the
 * autotuner in phinfortran_gb300/autotune.py).  panel: width of the panels
 * of the blocked Gauss-Jordan inverse (4, 8, 16 or 32; narrowed further
 * when a panel does not fit in shared memory); batch: most points a batch
 * (1..256).  0 restores the built-in choice.  Process-wide; set it before
 * sizing the workspace, which depends on it.  pf_tiled_layout reports the
 * panel width and batch a call of that shape would use.
 */
int pf_tiled_set_tuning(int panel, int batch);
int pf_tiled_layout(int n, int nl, int nr, int npts, int arith, int* panel, int* batch);

/*
 * Batched FP64-grade complex GEMM on the tcgen05 tensor cores.  No
 * counterpart in the reference (it is the block product the large-block
 * transport path is built on, exported for drivers that keep their own
 * recursion, e.g. negf/lesser.f90:587-589, 608 or negf/surface.f90:488-497):
 *     C_b = alpha op(A_b) op(B_b) + beta C_b,   b = 0 .. batch-1,
 * op = 'N' or 'C' (conjugate transpose), complex(kind=8) column-major
 * device arrays, real alpha and beta, batch strides in complex elements
 * (0 shares an operand), 1 <= k <= 2048 (PF_ERR_SIZE above).  Every row
 * of op(A) and column of op(B) is scaled by a power of two and split into
 * nine 7-bit BF16 slices (63 bits); the slice products that matter are
 * summed exactly on the tensor cores (FP32 accumulation of integers below
 * 2^22) and assembled in FP64, so the result has the accuracy of an FP64
 * GEMM (error O(k 2^-55) |A| |B|).
 * work: pf_tc_zgemm_workspace_size bytes of device memory (a_shared /
 * b_shared: strideA / strideB == 0).  Synchronous on `stream`.
 */
size_t pf_tc_zgemm_workspace_size(int m, int n, int k, int batch,
                                  int a_shared, int b_shared);

int pf_tc_zgemm_dev(int transa, int transb, int m, int n, int k,
                    double alpha, const double* A, int lda, long long strideA,
                    const double* B, int ldb, long long strideB, double beta,
                    double* C, int ldc, long long strideC, int batch,
                    void* work, size_t work_bytes, void* stream);

/* Message for the last error of pf_tc_zgemm_dev. */
const char* pf_tc_last_error(void);

/*
 * Tight-binding H(k) blocks (replaces gen_ham / V_sk / V_term / onsite of
 * tb/hamiltonian.f90:28-519 as used by gen_ham_mpi; the reference builds the
 * dense norb x norb matrix, here only the blocks the transport entries
 * take).  Atoms are grouped into nblk layers by blk_atom[0..nblk]
 * (increasing atom boundaries); orbitals follow gen_ham's order (atom-major,
 * then the species' orbital list).  For every k (fractional, kfrac[nk][3],
 * Cartesian k = kfrac . recivec) `out` receives, as interleaved complex
 * column-major blocks, first H_{I,I} for I = 0..nblk-1, then H_{I,I+1} for
 * I = 0..nblk-2, of the Hermitised matrix 0.5 (H + H^H).
 *   pos[natoms][3]   positions in Angstrom and r_d in metres, as the
 *                    reference holds them (V_term = V (r_d / |r| / 1e-10)^Vn),
 *                    species[natoms] 0-based
 *   orb_codes[nspecies][PF_TB_MAX_ORB]: 0 s, 1 px, 2 py, 3 pz, 4 dxy,
 *                    5 dyz, 6 dxz, 7 dx2-y2, 8 dz2, 9 s*
 *   V, Vn[nspecies][nspecies][4][4][4] (C order; principal numbers s 1, p 2,
 *                    d 3, s* 4; type 1 onsite, 2 sigma, 3 pi, 4 delta),
 *   r_d[nspecies][nspecies], latvec / recivec rows = vectors.
 * Host pointers; synchronous.
 */
#define PF_TB_MAX_ORB 10

int pf_tb_hk_blocks(int natoms, const double* pos, const int* species,
                    int nspecies, const int* norb_species, const int* orb_codes,
                    const double* V, const double* Vn, const double* r_d,
                    const double* latvec, const double* recivec,
                    double r_cutoff, int nk, const double* kfrac, int nblk,
                    const int* blk_atom, double* out);

/* Message for the last error of pf_tb_hk_blocks. */
const char* pf_tb_last_error(void);

/* ---------------------------------------------------------------------------
 * Binary force-constant (full-Hamiltonian) phonon path.
 *
 * pf_gen_dyn replaces gen_dyn_mpi (negf/dyn.f90:7-37 -> gen_dyn :39-150) and,
 * called with the lead tables and nz = 1, gen_dyn_lead_mpi
 * (negf/dyn.f90:152-187 -> gen_dyn_lead :190-312): the dense norb x norb
 * dynamical matrix, norb = 3 natoms, in THz^2,
 *   D(a i, b j) = sum over the entries of (a, b) of
 *                 fc(3 r(a) + i, 3 idx + j) exp(i dr . k) / sqrt(m_a m_b)
 * Hermitised (0.5 (D + D^H)) when `hermitize` is nonzero (gen_dyn, and the
 * in-layer matrix of gen_dyn_lead; its coupling matrix is not).  The entries
 * are the reference's reduced tables as the driver holds them
 * (negf/phinfortran.f90:655-683):
 *   num_mat[natoms x natoms]     Fortran column-major, num_mat(a+1, b+1) at
 *                                a + b*natoms; the entries run over (a, b)
 *                                row-major as the reference flattens them
 *   idx_mat_red[nent]            1-based fc column atoms
 *   dist_mat_red[nent x 3]       column-major (component c of entry e at
 *                                e + c*nent), Angstrom
 *   force_constant[fc_rows x fc_cols] column-major, eV/A^2, fc_rows = 3 n_uc
 *   mass[natoms]                 amu (mass_no of each atom's species)
 *   recivec[3][3]                rows = reciprocal vectors, kpoints[nq][3]
 *                                fractional (k = kpoint . recivec)
 * Atom a's fc row atom follows the z-slice order of negf/dyn.f90:95-103
 * (natoms = nbx*nby*n_uc, n_uc a multiple of nz).  Ham receives nq
 * column-major complex matrices.  Host pointers; synchronous.
 */
int pf_gen_dyn(int natoms, int nbx, int nby, int n_uc, int nz, int fc_rows,
               int fc_cols, const double* force_constant, const int* num_mat,
               int nent, const int* idx_mat_red, const double* dist_mat_red,
               const double* mass, const double* recivec, int nq,
               const double* kpoints, int hermitize, double* Ham);

/* The same on device buffers with the tables already packed: npairs atom
 * pairs (pair_a, pair_b 0-based) whose entries are pair_off[p] ..
 * pair_off[p+1]-1 of ent_idx (0-based fc column atom) and ent_dr[nent][3];
 * row_atom[natoms] the fc row atom of each atom, kcart[nq][3] Cartesian.
 * H receives nq column-major norb x norb complex matrices.  Asynchronous on
 * `stream`. */
int pf_gen_dyn_dev(int natoms, int fc_rows, const double* force_constant,
                   int npairs, const int* pair_a, const int* pair_b,
                   const int* pair_off, const int* ent_idx,
                   const double* ent_dr, const int* row_atom,
                   const double* mass, int nq, const double* kcart,
                   int hermitize, double* H, void* stream);

/* Block set of the tdb transport entries taken from nq dense matrices
 * (column-major norb x norb complex, device) as the full-Hamiltonian path
 * slices them: the left lead cell next to the device at rows n_buffer_l+nl
 * .. n_buffer_l+2nl-1 (Haml, and Hamlv = the block from the outer cell),
 * negf/surface.f90:170-198; the device layers from layer_start (device
 * int[L+1], orbital offsets from n_buffer_l+2nl; negf/device.f90:323-500,
 * the partition of blockwise_setup, :11-249); the right cells mirrored.
 * Every device block is zero-padded to n x n (padding rows/columns of the
 * couplings are zero, so the transmission is unchanged).  Outputs are the
 * device arrays of pf_transport_tdb_dev with a leading k axis.  *bad (device)
 * is set when a slice leaves the matrix.  Asynchronous on `stream`. */
int pf_dense_to_tdb_dev(int norb, int nq, const double* H, int nl, int nr,
                        int n_buffer_l, int n_buffer_r, int L,
                        const int* layer_start, int n, double* HL,
                        double* HLv, double* HR, double* HRv, double* Hd,
                        double* Hdv, double* Hld, double* Hrd, int* bad,
                        void* stream);

/* Message for the last error of the full-Hamiltonian entries. */
const char* pf_fullh_last_error(void);

/* ---------------------------------------------------------------------------
 * Buttiker probes (buttiker = 1): per point, get_G_full_tdb with the probe
 * self-energies (negf/lesser.f90:475-680) and get_G_lesser_tdb
 * (negf/lesser.f90:1199-1503), i.e. the bodies of get_G_full_tdb_mpi +
 * get_G_lesser_tdb_mpi (negf/phinfortran.f90:1204-1236) for a batch of
 * points.  Blocks as pf_transport_tdb (host pointers, n, nl, nr <= 48,
 * L >= 2).  Per point p and layer i (row-major [p][i], complex interleaved
 * where marked):
 *   sigw, dsigw [npts][L] complex: sigma_w(i, ie) and dsigma_wdt(i, ie) of
 *                set_sigma_bp_w (negf/lesser.f90:12-45) at the point's energy
 *   f, df [npts][L]: bose_einstein / dbosedT (negf/util.f90:987-1013) at
 *                sqrt(E) and the probe temperatures; fL, fR [npts] the leads'
 *   first [npts]: nonzero at the zero-frequency point (ie == 1), may be null
 * Outputs: transl [npts]; flux_i [npts][L], A_sum [npts][L] (Tr A_i),
 * Gn_i [npts][L] (Tr Gn_i), flux_left, flux_right [npts] (complex, as the
 * reference's arrays); jac [npts][L][L] complex, jac[p][i][j] = the
 * reference's jacobian(nn, ie, i, j).  Synchronous. */
int pf_buttiker_tdb(int n, int nl, int nr, int L, int nq, const double* HL,
                    const double* HLv, const double* HR, const double* HRv,
                    const double* Hd, const double* Hdv, const double* Hld,
                    const double* Hrd, int npts, const double* E,
                    const int* qidx, const int* first, const double* sigw,
                    const double* dsigw, const double* f, const double* df,
                    const double* fL, const double* fR, double eta,
                    double eta0, double dev_factor, double convergence,
                    int max_iter, double* transl, double* flux_i, double* jac,
                    double* A_sum, double* Gn_i, double* flux_left,
                    double* flux_right, int* status);

/* Message for the last error of pf_buttiker_tdb. */
const char* pf_buttiker_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* PHINFORTRAN_GB300_H */
