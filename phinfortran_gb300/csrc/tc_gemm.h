// FP64-grade complex GEMM on the tcgen05 tensor cores (host interface).
//
//   C_b = alpha op(A_b) op(B_b) + beta C_b  [- H_b]  [+ z_b I]
//
// complex(kind=8) column-major operands, op = N or C (conjugate transpose),
// real alpha and beta, a batch of independent products (a stride of 0
// shares an operand across the batch).  The products are formed from
// exact BF16 slice products (see tc_abi.cu), so the result carries the
// accuracy of an FP64 GEMM (about 2^-55 of |A| |B| per term), not that of
// the BF16 inputs.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace pf {
namespace tc {

// Bits per slice, slices per operand, and the largest pair sum s + t (1-based)
// whose products are accumulated exactly and drained into a 64-bit fixed
// point sum; pairs with s + t > kTopD go into one FP32 accumulator (their
// weight is at most 2^-49 of the leading pair's).  The tensor cores' FP32
// sums are not correctly rounded: a long chain of small addends drifts by
// about 2^-40 of the accumulator (measured), so only pairs that light may
// share the inexact accumulator.
constexpr int kBeta = 7;
constexpr int kSlices = 8;   // the 32-wide CTA-level products (tc_small.cuh)
constexpr int kSlicesL = 9;  // the batched large products (tc_abi.cu): 63-bit fixed point
constexpr int kTopD = 6;
constexpr int kBM = 128;     // rows of the real product per CTA (TMEM lanes)
constexpr int kBN = 64;      // columns per CTA
constexpr int kKStep = 64;   // K per TMA box (one 128-byte swizzle row of BF16)
constexpr int kChunk = 256;  // K per exact accumulation chain: 127^2 * 256 < 2^22
constexpr int kMaxK = 2048;  // largest complex K of the large products (16 chunks of the real K)

struct ZgemmArgs {
  int m, n, k;                 // op(A) is m x k, op(B) is k x n (complex)
  const void* A;               // double2
  int lda;
  long long sA;                // batch stride (complex elements), 0: shared
  bool ca;                     // op(A) = A^H
  const void* B;
  int ldb;
  long long sB;
  bool cb;
  void* C;                     // double2
  int ldc;
  long long sC;
  double alpha, beta;
  int batch;
  const int* active;           // per batch element (nullable): 0 -> skip
  const void* zdiag;           // per batch element z (double2, nullable): C += z I
  const void* H;               // nullable: C -= H_b
  int ldh;
  long long sH;
};

// Workspace bytes for the slices and exponents of one call of this shape.
size_t zgemm_workspace(int m, int n, int k, int batch, bool a_shared, bool b_shared);

// Launches the slicing and product kernels on `stream`.  Returns
// cudaSuccess or the first launch error; `err` (device int, nullable) gets
// bit 1 when a pipeline wait in the product kernel gave up (its outputs are
// then not written).
cudaError_t zgemm(const ZgemmArgs& g, void* work, size_t work_bytes, int* err, cudaStream_t stream);

// True when the driver provides cuTensorMapEncodeTiled (fetched through the
// runtime's driver entry point; the library does not link libcuda).
bool tma_available();

}  // namespace tc
}  // namespace pf
