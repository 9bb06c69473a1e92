// FP64 instantiation of the adjoint (gradient) kernel.
#include "grad_impl.cuh"

namespace pfgrad {

int grid_fp64(const GLayout& lay, int npts) { return grad_grid_r<double>(lay, npts); }

void launch_fp64(int grid, const GLayout& lay, const pf::System<double>& sys, const pf::Points& pts,
                 const pf::Params& P, const double* weights, const pf::Outputs& out, const pf::GradOut& go,
                 char* scratch, int* queue, cudaStream_t st) {
  grad_launch_r<double>(grid, lay, sys, pts, P, weights, out, go, scratch, queue, st);
}

}  // namespace pfgrad
