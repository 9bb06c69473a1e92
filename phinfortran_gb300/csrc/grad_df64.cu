// Double-float instantiation of the adjoint (gradient) kernel: every block
// product, inversion and decimation step in (hi, lo) float pairs on the
// FP32 pipe (about 48 significant bits); the sensitivities accumulate in
// FP64 through atomics.
#include "grad_impl.cuh"

namespace pfgrad {

namespace {
__global__ void to_df64_kernel(const double* __restrict__ src, pf::df64* __restrict__ dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = pf::df64(src[i]);
}
}  // namespace

int grid_df64(const GLayout& lay, int npts) { return grad_grid_r<pf::df64>(lay, npts); }

void launch_df64(int grid, const GLayout& lay, const pf::System<double>& sys, pf::df64* dst, const pf::Points& pts,
                 const pf::Params& P, const double* weights, const pf::Outputs& out, const pf::GradOut& go,
                 char* scratch, int* queue, cudaStream_t st) {
  const size_t nq = sys.nq, n = sys.n, nl = sys.nl, nr = sys.nr, L = sys.L;
  const size_t sizes[8] = {nq * nl * nl, nq * nl * nl, nq * nr * nr, nq * nr * nr,
                           nq * L * n * n, nq * (L > 1 ? L - 1 : 0) * n * n, nq * nl * n, nq * nr * n};
  const cx<double>* srcs[8] = {sys.HL, sys.HLv, sys.HR, sys.HRv, sys.Hd, sys.Hdv, sys.Hld, sys.Hrd};
  const cx<pf::df64>* outs[8];
  pf::df64* d = dst;
  for (int k = 0; k < 8; ++k) {
    outs[k] = reinterpret_cast<const cx<pf::df64>*>(d);
    const size_t nd = 2 * sizes[k];
    if (nd) to_df64_kernel<<<(unsigned)((nd + 255) / 256 < 4096 ? (nd + 255) / 256 : 4096), 256, 0, st>>>(
        reinterpret_cast<const double*>(srcs[k]), d, nd);
    d += nd;
  }
  pf::System<pf::df64> s2;
  s2.n = sys.n;
  s2.nl = sys.nl;
  s2.nr = sys.nr;
  s2.L = sys.L;
  s2.nq = sys.nq;
  s2.HL = outs[0];
  s2.HLv = outs[1];
  s2.HR = outs[2];
  s2.HRv = outs[3];
  s2.Hd = outs[4];
  s2.Hdv = outs[5];
  s2.Hld = outs[6];
  s2.Hrd = outs[7];
  grad_launch_r<pf::df64>(grid, lay, s2, pts, P, weights, out, go, scratch, queue, st);
}

}  // namespace pfgrad
