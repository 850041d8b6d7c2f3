// Double-float arithmetic ("dd"): a real held as an unevaluated sum hi + lo
// of two FP32 numbers with |lo| <= ulp(hi)/2, giving about 48 significant
// bits on the FP32 pipes.  On GB300 the FP32 pipes are 58x wider than the
// FP64 pipe (measured 69.9 vs 1.20 TFLOP/s), so transforms in this format
// run several times faster than in FP64 while keeping errors near 1e-14.
//
// Building blocks are the error-free transformations of Knuth (two-sum) and
// Dekker (fast two-sum), with the product error taken from an FMA; the
// addition is the accurate variant that normalises both the high and the low
// sums (Hida, Li & Bailey, "Library for double-double and quad-double
// arithmetic", 2007, Algorithm 6 adapted to FP32 components).
#pragma once

#include <cuda_runtime.h>

namespace chgpu {

struct dd {
  float hi, lo;
  __host__ __device__ constexpr dd() : hi(0.f), lo(0.f) {}
  __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
  // split of a double: exact when the double's exponent fits FP32's range
  __host__ __device__ dd(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ dd two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return dd(s, e);
}
__device__ __forceinline__ dd fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return dd(s, e);
}
__device__ __forceinline__ dd operator+(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  dd t = two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = fast_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dd operator-(dd a) { return dd(-a.hi, -a.lo); }
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }
__device__ __forceinline__ dd operator*(dd a, dd b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ bool operator<(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(dd a, dd b) { return b < a; }
__device__ __forceinline__ bool operator==(dd a, dd b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ dd fabs(dd a) { return a.hi < 0.f ? -a : a; }
__device__ __forceinline__ dd max(dd a, dd b) { return (a < b) ? b : a; }
__device__ __forceinline__ bool isfinite(dd a) { return ::isfinite(a.hi) && ::isfinite(a.lo); }

// complex double-float: 16 bytes, like double2
struct __align__(16) cdd {
  dd x, y;
};

}  // namespace chgpu
