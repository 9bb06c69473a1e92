// extern "C" boundary of the GB300 NEGF transport engine.
//
// The entry points replace the per-(ie,ik) Fortran calls of the tdb
// transport loop (negf/phinfortran.f90:1196-1213):
//   surface_green_tdb_mpi  (negf/surface.f90:344-383)
//   get_G_full_tdb_mpi     (negf/lesser.f90:100-157)
// batched over every (omega, q) point of a shard.  Matrices are the
// reference's complex(kind=8) column-major blocks; all pointers are plain
// double* to interleaved (re, im) pairs.
//
// This unit holds the FP64 path, the host-pointer entries and the
// allocation-free entry; the mixed-precision pipeline is in negf_mixed.cu.
#include <mutex>
#include <vector>

#include "negf_common.cuh"

thread_local char pf_negf_err[512] = "";

namespace {
template <typename R>
__device__ pf::Ctx<R> make_ctx(const Layout& lay, char* gscr_base) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pf::Ctx<R> c;
  cx<R>* s = reinterpret_cast<cx<R>*>(smem_raw);
  for (int i = 0; i < pf::NSM; ++i) c.sm[i] = s + i * lay.mat;
  // tail: 32 reduction words, then the pivot row/column vectors, then ints
  unsigned char* tail = reinterpret_cast<unsigned char*>(s + pf::NSM * lay.mat);
  c.red = reinterpret_cast<double*>(tail);
  c.iw.rowk = reinterpret_cast<cx<R>*>(tail + 32 * sizeof(double));
  c.iw.colk = c.iw.rowk + lay.m;
  int* ip = reinterpret_cast<int*>(c.iw.colk + lay.m);
  c.iw.perm = ip;
  c.iw.flag = ip + lay.m;
  cx<R>* g = reinterpret_cast<cx<R>*>(gscr_base) + (size_t)blockIdx.x * pf::NG * lay.mat;
  for (int i = 0; i < pf::NG; ++i) c.gs[i] = g + i * lay.mat;
  c.ld = lay.ld;
  return c;
}

// Fused persistent kernel: each CTA pulls points from a device work queue,
// runs both lead decimations, the left-to-right sweep (and optionally the
// right-to-left one) and the Caroli traces, and retires the point.
template <typename R, int S>
__global__ void __launch_bounds__(kThreads) transport_kernel(pf::System<R> sys, pf::Points pts,
                                                             pf::Params P, pf::Outputs out, Layout lay,
                                                             char* gscr, int* queue) {
  pf::Ctx<R> c = make_ctx<R>(lay, gscr);
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
    int st = pf::lead_pair<R, S>(c, sys, q, E, P, &itl, &itr);
    const double eps = E * P.eta + P.eta0;
    const cx<R> zD = pf::mk<R>(R(E), R(P.dev_factor * eps));
    double tl = 0, tr = 0;
    st |= pf::sweep_lr<R, S>(c, sys, q, zD, &tl);
    if (P.want_transr) st |= pf::sweep_rl<R, S>(c, sys, q, zD, &tr);
    if (threadIdx.x == 0) {
      const bool zero = pts.zero_flag && pts.zero_flag[p];
      double a = (double)tl, b = (double)tr;
      // lesser.f90:795-807: values below 1e-60 (a NaN is not) become 0; ie==1 -> 0
      if (zero || a < 1.0e-60) a = 0.0;
      if (zero || b < 1.0e-60) b = 0.0;
      out.transl[p] = a;
      if (out.transr) out.transr[p] = P.want_transr ? b : 0.0;
      out.status[p] = st;
      if (out.iters) {
        out.iters[2 * p] = itl;
        out.iters[2 * p + 1] = itr;
      }
    }
    __syncthreads();
  }
}

template <typename R, int S>
int grid_for(const Layout& lay, int npts) {
  auto k = transport_kernel<R, S>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.smem) != cudaSuccess)
    return -1;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, lay.smem) != cudaSuccess) return -1;
  if (per_sm < 1) return -1;
  DevInfo d = device_info();
  int g = d.sms * per_sm;
  return g < npts ? g : npts;
}

template <typename R>
int launch_transport(const pf::System<R>& sys, const pf::Points& pts, const pf::Params& P,
                     const pf::Outputs& out, void* work, size_t work_bytes, cudaStream_t stream) {
  const Layout lay = make_layout<R>(sys.n, sys.nl, sys.nr);
  DevInfo d = device_info();
  if (lay.smem > d.smem_optin) return set_err(PF_ERR_SIZE, "pf: working set exceeds shared memory");
  if (pts.npts == 0) return PF_SUCCESS;
  const int S = (lay.m + 31) / 32;
  int grid = (S == 1) ? grid_for<R, 1>(lay, pts.npts) : grid_for<R, 2>(lay, pts.npts);
  if (grid <= 0) return set_err(PF_ERR_SIZE, "pf: kernel does not fit on the device");
  const size_t mir = ((size_t)sys.nq * sizeof(int) + 255) & ~(size_t)255;
  const size_t need = 256 + mir + (size_t)grid * lay.per_cta_bytes;
  if (!work || work_bytes < need) return set_err(PF_ERR_ARG, "pf: workspace too small");
  int* queue = reinterpret_cast<int*>(work);
  int* mirror = reinterpret_cast<int*>(reinterpret_cast<char*>(work) + 256);
  char* gscr = reinterpret_cast<char*>(work) + 256 + mir;
  PF_CUDA(cudaMemsetAsync(queue, 0, sizeof(int), stream));
  pf::Params P2 = P;
  if (sys.nl == sys.nr) {
    lead_mirror_kernel<<<sys.nq, 256, 0, stream>>>(reinterpret_cast<const double*>(sys.HL),
                                                   reinterpret_cast<const double*>(sys.HLv),
                                                   reinterpret_cast<const double*>(sys.HR),
                                                   reinterpret_cast<const double*>(sys.HRv), 2 * sys.nl * sys.nl,
                                                   sys.nq, mirror);
    P2.lead_mirror = mirror;
  } else {
    P2.lead_mirror = nullptr;
  }
  if (S == 1)
    transport_kernel<R, 1><<<grid, kThreads, lay.smem, stream>>>(sys, pts, P2, out, lay, gscr, queue);
  else
    transport_kernel<R, 2><<<grid, kThreads, lay.smem, stream>>>(sys, pts, P2, out, lay, gscr, queue);
  PF_CUDA(cudaGetLastError());
  return PF_SUCCESS;
}

template <typename R>
size_t workspace_bytes(int n, int nl, int nr, int nq, int npts) {
  const Layout lay = make_layout<R>(n, nl, nr);
  const int S = (lay.m + 31) / 32;
  int grid = (S == 1) ? grid_for<R, 1>(lay, npts > 0 ? npts : 1) : grid_for<R, 2>(lay, npts > 0 ? npts : 1);
  if (grid <= 0) return 0;
  return 256 + (((size_t)nq * sizeof(int) + 255) & ~(size_t)255) + (size_t)grid * lay.per_cta_bytes;
}

pf::System<double> make_sys(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                            const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                            const double* Hld, const double* Hrd) {
  pf::System<double> s;
  s.n = n;
  s.nl = nl;
  s.nr = nr;
  s.L = L;
  s.nq = nq;
  s.HL = reinterpret_cast<const cx<double>*>(HL);
  s.HLv = reinterpret_cast<const cx<double>*>(HLv);
  s.HR = reinterpret_cast<const cx<double>*>(HR);
  s.HRv = reinterpret_cast<const cx<double>*>(HRv);
  s.Hd = reinterpret_cast<const cx<double>*>(Hd);
  s.Hdv = reinterpret_cast<const cx<double>*>(Hdv);
  s.Hld = reinterpret_cast<const cx<double>*>(Hld);
  s.Hrd = reinterpret_cast<const cx<double>*>(Hrd);
  return s;
}

// Grow-only device buffers used by the host-pointer entry point.
struct HostStage {
  std::mutex mu;
  void* buf = nullptr;
  size_t cap = 0;
  int dev = -1;
};
HostStage g_stage;


// ===========================================================================
// Allocation-free variant of the FP64 transport entry.
//
// Some callers cannot hand this library a device workspace: host codes that
// reserve the GPU's memory up front through their own allocator and forbid
// any later cudaMalloc (or cannot expose a device pointer for scratch at
// the call site).  For them pf_transport_tdb_noalloc keeps its scratch --
// the work-queue counter, the lead-mirror flags and the per-CTA matrices of
// the persistent kernel -- in the file-scope array below.  Every GPU that
// loads the library holds PF_NOALLOC_SCRATCH_BYTES of it until the process
// exits.  All calls share the array and it keeps the contents of the last
// call: the queue counter is cleared and the mirror flags rewritten on
// every call, and calls whose kernels overlap on the GPU race on it.
// ===========================================================================
static __device__ __align__(256) unsigned char g_noalloc_scratch[PF_NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mu;
struct NoallocSlot {
  void* ptr;
  unsigned long long ctx_id;  // the CUDA context the address belongs to
};
NoallocSlot g_noalloc_slot[128] = {};

// Driver calls that identify the current context, fetched through the
// runtime (the library does not link libcuda itself).
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

int current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
      (void)cudaGetLastError();
      return set_err(PF_ERR_CUDA, "pf_transport_tdb_noalloc: driver context queries unavailable");
    }
    get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  void* ctx = nullptr;
  *id = 0;
  if (get_current(&ctx) != 0) return set_err(PF_ERR_CUDA, "pf_transport_tdb_noalloc: cuCtxGetCurrent failed");
  if (ctx && get_id(ctx, id) != 0) return set_err(PF_ERR_CUDA, "pf_transport_tdb_noalloc: cuCtxGetId failed");
  return PF_SUCCESS;
}

// Device address of the static scratch for the current device.  Set-up,
// once per device: the first call on a device (with that device current)
// resolves it with cudaGetSymbolAddress; later calls reuse it.  The address
// is tied to the device's CUDA context: after a device reset the next call
// runs in a new context (a new context id) and resolves the address again,
// since the reloaded module may place the array elsewhere.  The set-up call
// must not be captured into a CUDA graph (it may load the module): a call
// that would need the set-up during stream capture is refused.
int noalloc_scratch(cudaStream_t stream, void** out) {
  int dev = 0;
  PF_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 128) return set_err(PF_ERR_ARG, "pf: device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  unsigned long long id = 0;
  int rc = current_context_id(&id);
  if (rc != PF_SUCCESS) return rc;
  NoallocSlot& slot = g_noalloc_slot[dev];
  if (id == 0 || !slot.ptr || slot.ctx_id != id) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const cudaError_t qe = cudaStreamIsCapturing(stream, &cap);
    if (qe != cudaSuccess) (void)cudaGetLastError();
    if (qe != cudaSuccess || cap != cudaStreamCaptureStatusNone)
      return set_err(PF_ERR_ARG,
                     "pf_transport_tdb_noalloc: first call on this device (or after a device reset) made "
                     "during stream capture; make one call outside capture first");
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_err(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    rc = current_context_id(&id);  // the lookup creates the context when none was current
    if (rc != PF_SUCCESS) return rc;
    slot.ptr = ptr;
    slot.ctx_id = id;
  }
  *out = slot.ptr;
  return PF_SUCCESS;
}

// Same launch as launch_transport, with the persistent grid capped so that
// the per-CTA scratch fits in the static array.
int launch_transport_noalloc(const pf::System<double>& sys, const pf::Points& pts, const pf::Params& P,
                             const pf::Outputs& out, cudaStream_t stream) {
  const Layout lay = make_layout<double>(sys.n, sys.nl, sys.nr);
  DevInfo d = device_info();
  if (lay.smem > d.smem_optin) return set_err(PF_ERR_SIZE, "pf: working set exceeds shared memory");
  const size_t mir = ((size_t)sys.nq * sizeof(int) + 255) & ~(size_t)255;
  const size_t fixed = 256 + mir;
  if (fixed + lay.per_cta_bytes > (size_t)PF_NOALLOC_SCRATCH_BYTES)
    return set_err(PF_ERR_SIZE,
                   "pf_transport_tdb_noalloc: problem needs more scratch than the static maximum "
                   "PF_NOALLOC_SCRATCH_BYTES (too many q points or too large blocks)");
  if (pts.npts == 0) return PF_SUCCESS;
  const int S = (lay.m + 31) / 32;
  int grid = (S == 1) ? grid_for<double, 1>(lay, pts.npts) : grid_for<double, 2>(lay, pts.npts);
  if (grid <= 0) return set_err(PF_ERR_SIZE, "pf: kernel does not fit on the device");
  const size_t cap = ((size_t)PF_NOALLOC_SCRATCH_BYTES - fixed) / lay.per_cta_bytes;
  if ((size_t)grid > cap) grid = (int)cap;
  void* base = nullptr;
  int rc = noalloc_scratch(stream, &base);
  if (rc != PF_SUCCESS) return rc;
  int* queue = reinterpret_cast<int*>(base);
  int* mirror = reinterpret_cast<int*>(reinterpret_cast<char*>(base) + 256);
  char* gscr = reinterpret_cast<char*>(base) + fixed;
  PF_CUDA(cudaMemsetAsync(queue, 0, sizeof(int), stream));
  pf::Params P2 = P;
  if (sys.nl == sys.nr) {
    lead_mirror_kernel<<<sys.nq, 256, 0, stream>>>(reinterpret_cast<const double*>(sys.HL),
                                                   reinterpret_cast<const double*>(sys.HLv),
                                                   reinterpret_cast<const double*>(sys.HR),
                                                   reinterpret_cast<const double*>(sys.HRv), 2 * sys.nl * sys.nl,
                                                   sys.nq, mirror);
    P2.lead_mirror = mirror;
  } else {
    P2.lead_mirror = nullptr;
  }
  if (S == 1)
    transport_kernel<double, 1><<<grid, kThreads, lay.smem, stream>>>(sys, pts, P2, out, lay, gscr, queue);
  else
    transport_kernel<double, 2><<<grid, kThreads, lay.smem, stream>>>(sys, pts, P2, out, lay, gscr, queue);
  PF_CUDA(cudaGetLastError());
  return PF_SUCCESS;
}
}  // namespace

extern "C" int pf_transport_tdb_dev(int, int, int, int, int, const double*, const double*, const double*,
                                    const double*, const double*, const double*, const double*, const double*, int,
                                    const double*, const int*, const int*, double, double, double, double, int, int,
                                    double*, double*, int*, int*, void*, size_t, void*);
extern "C" int pf_transport_tdb_mixed_dev(int, int, int, int, int, const double*, const double*, const double*,
                                          const double*, const double*, const double*, const double*,
                                          const double*, int, const double*, const int*, const int*, double,
                                          double, double, double, int, int, double*, int*, int*, void*, size_t,
                                          void*);
namespace {
int host_run(bool mixed, int refine_iters, int n, int nl, int nr, int L, int nq, const double* HL,
             const double* HLv, const double* HR, const double* HRv, const double* Hd, const double* Hdv,
             const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
             const int* zero_flag, double eta, double eta0, double dev_factor, double convergence, int max_iter,
             int want_transr, double* transl, double* transr, int* status, int* iters) {
  int rc = check_dims(n, nl, nr, L, nq, npts);
  if (rc != PF_SUCCESS) return rc;
  if (!E || !transl || !status || (want_transr && !transr))
    return set_err(PF_ERR_ARG, "pf: null energy/output pointer");
  if (npts == 0) return PF_SUCCESS;
  std::lock_guard<std::mutex> lock(g_stage.mu);
  const size_t c16 = 16;
  const size_t b_HL = (size_t)nq * nl * nl * c16, b_HR = (size_t)nq * nr * nr * c16;
  const size_t b_Hd = (size_t)nq * L * n * n * c16, b_Hdv = (size_t)nq * (L - 1) * n * n * c16;
  const size_t b_Hld = (size_t)nq * nl * n * c16, b_Hrd = (size_t)nq * nr * n * c16;
  const size_t b_E = (size_t)npts * 8, b_i = (size_t)npts * 4;
  const size_t ws = mixed ? pf_transport_tdb_mixed_workspace_size(n, nl, nr, L, nq, npts)
                          : workspace_bytes<double>(n, nl, nr, nq, npts);
  if (ws == 0) return set_err(PF_ERR_SIZE, "pf: kernel does not fit on the device");
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t total = al(b_HL) * 2 + al(b_HR) * 2 + al(b_Hd) + al(b_Hdv) + al(b_Hld) + al(b_Hrd) + al(b_E) +
                       al(b_i) * 2 + al(b_E) * 2 + al(b_i) + al(2 * b_i) + al(ws);
  int dev = 0;
  PF_CUDA(cudaGetDevice(&dev));
  if (g_stage.cap < total || g_stage.dev != dev) {
    if (g_stage.buf) cudaFree(g_stage.buf);
    g_stage.buf = nullptr;
    g_stage.cap = 0;
    PF_CUDA(cudaMalloc(&g_stage.buf, total));
    g_stage.cap = total;
    g_stage.dev = dev;
  }
  char* p = reinterpret_cast<char*>(g_stage.buf);
  auto take = [&](size_t b) {
    char* r = p;
    p += al(b);
    return r;
  };
  double* dHL = (double*)take(b_HL);
  double* dHLv = (double*)take(b_HL);
  double* dHR = (double*)take(b_HR);
  double* dHRv = (double*)take(b_HR);
  double* dHd = (double*)take(b_Hd);
  double* dHdv = (double*)take(b_Hdv);
  double* dHld = (double*)take(b_Hld);
  double* dHrd = (double*)take(b_Hrd);
  double* dE = (double*)take(b_E);
  int* dq = (int*)take(b_i);
  int* dz = (int*)take(b_i);
  double* dTL = (double*)take(b_E);
  double* dTR = (double*)take(b_E);
  int* dst = (int*)take(b_i);
  int* dit = (int*)take(2 * b_i);
  void* dws = take(ws);
  cudaStream_t s = 0;
  PF_CUDA(cudaMemcpyAsync(dHL, HL, b_HL, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dHLv, HLv, b_HL, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dHR, HR, b_HR, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dHRv, HRv, b_HR, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dHd, Hd, b_Hd, cudaMemcpyHostToDevice, s));
  if (L > 1) PF_CUDA(cudaMemcpyAsync(dHdv, Hdv, b_Hdv, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dHld, Hld, b_Hld, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dHrd, Hrd, b_Hrd, cudaMemcpyHostToDevice, s));
  PF_CUDA(cudaMemcpyAsync(dE, E, b_E, cudaMemcpyHostToDevice, s));
  if (qidx) PF_CUDA(cudaMemcpyAsync(dq, qidx, b_i, cudaMemcpyHostToDevice, s));
  if (zero_flag) PF_CUDA(cudaMemcpyAsync(dz, zero_flag, b_i, cudaMemcpyHostToDevice, s));
  if (mixed)
    rc = pf_transport_tdb_mixed_dev(n, nl, nr, L, nq, dHL, dHLv, dHR, dHRv, dHd, dHdv, dHld, dHrd, npts, dE,
                                    qidx ? dq : nullptr, zero_flag ? dz : nullptr, eta, eta0, dev_factor,
                                    convergence, max_iter, refine_iters, dTL, dst, dit, dws, ws, s);
  else
    rc = pf_transport_tdb_dev(n, nl, nr, L, nq, dHL, dHLv, dHR, dHRv, dHd, dHdv, dHld, dHrd, npts, dE,
                              qidx ? dq : nullptr, zero_flag ? dz : nullptr, eta, eta0, dev_factor, convergence,
                              max_iter, want_transr, dTL, dTR, dst, dit, dws, ws, s);
  if (rc != PF_SUCCESS) return rc;
  PF_CUDA(cudaMemcpyAsync(transl, dTL, b_E, cudaMemcpyDeviceToHost, s));
  if (want_transr) PF_CUDA(cudaMemcpyAsync(transr, dTR, b_E, cudaMemcpyDeviceToHost, s));
  PF_CUDA(cudaMemcpyAsync(status, dst, b_i, cudaMemcpyDeviceToHost, s));
  if (iters) PF_CUDA(cudaMemcpyAsync(iters, dit, 2 * b_i, cudaMemcpyDeviceToHost, s));
  PF_CUDA(cudaStreamSynchronize(s));
  int any = 0;
  for (int i = 0; i < npts; ++i) any |= status[i];
  if (any) {
    snprintf(pf_negf_err, sizeof(pf_negf_err), "pf: point status flags 0x%x (1 singular, 2 nan, 4 not converged)", any);
    return PF_ERR_POINT;
  }
  return PF_SUCCESS;
}
}  // namespace

extern "C" {

const char* pf_last_error(void) { return pf_negf_err; }

int pf_version(void) { return PF_ABI_VERSION; }

size_t pf_transport_tdb_workspace_size(int n, int nl, int nr, int nq, int npts) {
  if (check_dims(n, nl, nr, 1, nq, npts) != PF_SUCCESS) return 0;
  return workspace_bytes<double>(n, nl, nr, nq, npts);
}

int pf_transport_tdb_dev(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                         const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                         const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                         const int* zero_flag, double eta, double eta0, double dev_factor, double convergence,
                         int max_iter, int want_transr, double* transl, double* transr, int* status,
                         int* iters, void* work, size_t work_bytes, void* stream) {
  int rc = check_dims(n, nl, nr, L, nq, npts);
  if (rc != PF_SUCCESS) return rc;
  if (!E || !transl || !status || (want_transr && !transr))
    return set_err(PF_ERR_ARG, "pf: null energy/output pointer");
  if (!HL || !HLv || !HR || !HRv || !Hd || !Hld || !Hrd || (L > 1 && !Hdv))
    return set_err(PF_ERR_ARG, "pf: null block pointer");
  if (max_iter <= 0) return set_err(PF_ERR_ARG, "pf: max_iter must be positive");
  pf::System<double> sys = make_sys(n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd);
  pf::Points pts{npts, E, qidx, zero_flag};
  pf::Params P{nullptr, eta, eta0, dev_factor, convergence, max_iter, want_transr};
  pf::Outputs out{transl, want_transr ? transr : nullptr, status, iters};
  return launch_transport<double>(sys, pts, P, out, work, work_bytes, (cudaStream_t)stream);
}


}  // extern "C"

extern "C" {

int pf_transport_tdb_mixed(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                           const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                           const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                           const int* zero_flag, double eta, double eta0, double dev_factor, double convergence,
                           int max_iter, int refine_iters, double* transl, int* status, int* iters) {
  return host_run(true, refine_iters, n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd, npts, E, qidx,
                  zero_flag, eta, eta0, dev_factor, convergence, max_iter, 0, transl, nullptr, status, iters);
}

int pf_transport_tdb(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv, const double* HR,
                     const double* HRv, const double* Hd, const double* Hdv, const double* Hld,
                     const double* Hrd, int npts, const double* E, const int* qidx, const int* zero_flag,
                     double eta, double eta0, double dev_factor, double convergence, int max_iter,
                     int want_transr, double* transl, double* transr, int* status, int* iters) {
  return host_run(false, 0, n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd, npts, E, qidx, zero_flag, eta,
                  eta0, dev_factor, convergence, max_iter, want_transr, transl, transr, status, iters);
}

int pf_transport_tdb_noalloc(int n, int nl, int nr, int L, int nq, const double* HL, const double* HLv,
                             const double* HR, const double* HRv, const double* Hd, const double* Hdv,
                             const double* Hld, const double* Hrd, int npts, const double* E, const int* qidx,
                             const int* zero_flag, double eta, double eta0, double dev_factor, double convergence,
                             int max_iter, int want_transr, double* transl, double* transr, int* status,
                             int* iters, void* stream) {
  int rc = check_dims(n, nl, nr, L, nq, npts);
  if (rc != PF_SUCCESS) return rc;
  if (!E || !transl || !status || (want_transr && !transr))
    return set_err(PF_ERR_ARG, "pf: null energy/output pointer");
  if (!HL || !HLv || !HR || !HRv || !Hd || !Hld || !Hrd || (L > 1 && !Hdv))
    return set_err(PF_ERR_ARG, "pf: null block pointer");
  if (max_iter <= 0) return set_err(PF_ERR_ARG, "pf: max_iter must be positive");
  pf::System<double> sys = make_sys(n, nl, nr, L, nq, HL, HLv, HR, HRv, Hd, Hdv, Hld, Hrd);
  pf::Points pts{npts, E, qidx, zero_flag};
  pf::Params P{nullptr, eta, eta0, dev_factor, convergence, max_iter, want_transr};
  pf::Outputs out{transl, want_transr ? transr : nullptr, status, iters};
  return launch_transport_noalloc(sys, pts, P, out, (cudaStream_t)stream);
}

}  // extern "C"
