// Double-float ("df64") real arithmetic on the FP32 pipe.
//
// A value is hi + lo with |lo| <= ulp(hi)/2, about 48 significant bits.
// GB300 executes FP32 about 67x faster than FP64, so df64 arithmetic built
// from error-free transformations runs several times faster than native
// FP64 while keeping ~1e-14 relative precision.
//
// The transformations are the classical ones of Dekker (1971) and Knuth
// (TAOCP vol. 2, 4.2.2):
//   TwoSum(a,b):      s = a+b, v = s-a, e = (a-(s-v)) + (b-v)      (exact)
//   QuickTwoSum(a,b): s = a+b, e = b-(s-a)   for |a| >= |b|       (exact)
//   TwoProd(a,b):     p = a*b, e = fma(a,b,-p)                      (exact)
// Every operation uses the _rn intrinsics so the compiler cannot contract
// or reassociate them.  Addition is the "sloppy" variant (one TwoSum): its
// error is bounded by ~2^-47 (|a|+|b|), the normwise bound dense linear
// algebra needs.
#pragma once
#include <cuda_runtime.h>

namespace pf {

struct df64 {
  float hi, lo;
  __host__ __device__ df64() : hi(0.f), lo(0.f) {}
  __host__ __device__ df64(float h, float l) : hi(h), lo(l) {}
  __device__ df64(double d) {
    hi = __double2float_rn(d);
    lo = __double2float_rn(d - (double)hi);
  }
  __device__ df64(int i) : hi((float)i), lo(0.f) {}
};

__device__ __forceinline__ df64 quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return df64(s, e);
}
__device__ __forceinline__ df64 two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
  return df64(s, e);
}
__device__ __forceinline__ df64 two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  return df64(p, e);
}

__device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return quick_two_sum(s.hi, e);
}
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + (-b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  df64 p = two_prod(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.lo, p.lo);
  e = __fmaf_rn(a.lo, b.hi, e);
  return quick_two_sum(p.hi, e);
}
// a*b + c with one rounding of the df64 product
__device__ __forceinline__ df64 fma(df64 a, df64 b, df64 c) {
  df64 p = two_prod(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.lo, p.lo);
  e = __fmaf_rn(a.lo, b.hi, e);
  df64 s = two_sum(p.hi, c.hi);
  const float t = __fadd_rn(s.lo, __fadd_rn(c.lo, e));
  return quick_two_sum(s.hi, t);
}
// 1/b by one Newton step from the float reciprocal: r = r0 + r0 (1 - b r0)
__device__ __forceinline__ df64 recip(df64 b) {
  const float r0 = __frcp_rn(b.hi);
  const df64 one(1.f, 0.f);
  const df64 r(r0, 0.f);
  const df64 e = one - b * r;
  return r + r * e;
}
__device__ __forceinline__ df64 operator/(df64 a, df64 b) {
  // q0 = a * (1/b), then one correction with the residual a - b q0
  const df64 r = recip(b);
  const df64 q0 = a * r;
  const df64 res = a - b * q0;
  return q0 + res * r;
}
__device__ __forceinline__ double to_d(df64 a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ double to_d(double a) { return a; }
__device__ __forceinline__ double to_d(float a) { return (double)a; }

// The df64 overloads below live in namespace pf and would hide the global
// double/float functions inside it, so forward those explicitly.
__device__ __forceinline__ double fabs(double a) { return ::fabs(a); }
__device__ __forceinline__ float fabs(float a) { return ::fabsf(a); }
__device__ __forceinline__ double fma(double a, double b, double c) { return ::fma(a, b, c); }
__device__ __forceinline__ float fma(float a, float b, float c) { return ::fmaf(a, b, c); }
__device__ __forceinline__ bool isfinite(double a) { return ::isfinite(a); }
__device__ __forceinline__ bool isfinite(float a) { return ::isfinite(a); }

__device__ __forceinline__ df64 fabs(df64 a) { return a.hi < 0.f ? -a : a; }
__device__ __forceinline__ bool isfinite(df64 a) { return ::isfinite(a.hi) && ::isfinite(a.lo); }
__device__ __forceinline__ bool operator>(df64 a, df64 b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__device__ __forceinline__ bool operator<(df64 a, df64 b) { return b > a; }
__device__ __forceinline__ bool operator>=(df64 a, df64 b) { return !(b > a); }
__device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ bool operator!=(df64 a, df64 b) { return !(a == b); }

__device__ __forceinline__ df64 shfl_r(df64 v, int src) {
  return df64(__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src));
}
__device__ __forceinline__ double shfl_r(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ float shfl_r(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// real-type conversions used by the mixed-precision stages
template <typename To>
__device__ __forceinline__ To conv(double v);
template <>
__device__ __forceinline__ double conv<double>(double v) { return v; }
template <>
__device__ __forceinline__ float conv<float>(double v) { return (float)v; }
template <>
__device__ __forceinline__ df64 conv<df64>(double v) { return df64(v); }

}  // namespace pf
