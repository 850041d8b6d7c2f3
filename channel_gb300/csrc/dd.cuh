// Double-float arithmetic ("dd"): a real held as an unevaluated sum hi + lo
// of two FP32 numbers with |lo| <= ulp(hi)/2, giving about 48 significant
// bits on the FP32 pipes.  On GB300 the FP32 pipes are 58x wider than the
// FP64 pipe (measured 69.9 vs 1.20 TFLOP/s), so transforms in this format
// run several times faster than in FP64 while keeping errors near 1e-14.
//
// Building blocks are the error-free transformations of Knuth (two-sum) and
// Dekker (fast two-sum), with the product error taken from an FMA (Dekker,
// "A floating-point technique for extending the available precision", 1971;
// error bounds in Joldes, Muller & Popescu, "Tight and rigorous error bounds
// for basic building blocks of double-word arithmetic", 2017).
#pragma once

#include <cuda_runtime.h>

namespace chgpu {

struct dd {
  float hi, lo;
  __host__ __device__ constexpr dd() : hi(0.f), lo(0.f) {}
  __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr explicit dd(float h) : hi(h), lo(0.f) {}
  // split of a double: exact when the double's exponent fits FP32's range
  __host__ __device__ explicit dd(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
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
// Dekker's addition ("sloppy" double-word add): the high parts added
// error-free, the low parts and the error summed in FP32, one
// renormalisation; 11 FP32 operations.  Its error is bounded relative to
// |a| + |b| (about 2^-46 of it), the same form as the error of an FP64
// addition of inputs that carry their own rounding.
__device__ __forceinline__ dd operator+(dd a, dd b) {
  const dd s = two_sum(a.hi, b.hi);
  const float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}
// Addition without the final renormalisation (8 FP32 operations): the high
// parts summed error-free, the low parts and the error in FP32.  For
// intermediate sums that only feed further arithmetic: the pair's low part
// may exceed half an ulp of its high part by a few ulps, which the next
// error-free sum of the high parts absorbs.
__device__ __forceinline__ dd add_nr(dd a, dd b) {
  const dd s = two_sum(a.hi, b.hi);
  return dd(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
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
__device__ __forceinline__ dd dd_abs(dd a) { return a.hi < 0.f ? -a : a; }
__device__ __forceinline__ dd dd_max(dd a, dd b) { return (a < b) ? b : a; }
__device__ __forceinline__ bool dd_isfinite(dd a) { return isfinite(a.hi) && isfinite(a.lo); }

// x1*y1 + x2*y2 with one renormalisation: both products exactly as
// hi-product + FMA error + cross terms, one two-sum of the high parts.
__device__ __forceinline__ dd dd_dot2(dd x1, dd y1, dd x2, dd y2) {
  const float p1 = __fmul_rn(x1.hi, y1.hi);
  float e1 = __fmaf_rn(x1.hi, y1.hi, -p1);
  e1 = __fmaf_rn(x1.hi, y1.lo, e1);
  e1 = __fmaf_rn(x1.lo, y1.hi, e1);
  const float p2 = __fmul_rn(x2.hi, y2.hi);
  float e2 = __fmaf_rn(x2.hi, y2.hi, -p2);
  e2 = __fmaf_rn(x2.hi, y2.lo, e2);
  e2 = __fmaf_rn(x2.lo, y2.hi, e2);
  dd s = two_sum(p1, p2);
  s.lo = __fadd_rn(s.lo, __fadd_rn(e1, e2));
  return fast_two_sum(s.hi, s.lo);
}

// the same without the final renormalisation, for products that feed only
// further sums
__device__ __forceinline__ dd dd_dot2_nr(dd x1, dd y1, dd x2, dd y2) {
  const float p1 = __fmul_rn(x1.hi, y1.hi);
  float e1 = __fmaf_rn(x1.hi, y1.hi, -p1);
  e1 = __fmaf_rn(x1.hi, y1.lo, e1);
  e1 = __fmaf_rn(x1.lo, y1.hi, e1);
  const float p2 = __fmul_rn(x2.hi, y2.hi);
  float e2 = __fmaf_rn(x2.hi, y2.hi, -p2);
  e2 = __fmaf_rn(x2.hi, y2.lo, e2);
  e2 = __fmaf_rn(x2.lo, y2.hi, e2);
  const dd s = two_sum(p1, p2);
  return dd(s.hi, __fadd_rn(s.lo, __fadd_rn(e1, e2)));
}

// complex double-float: 16 bytes, like double2
struct __align__(16) cdd {
  dd x, y;
};
// complex product in two fused dot products (38 FP32 operations instead of 68)
__device__ __forceinline__ cdd cmul(cdd a, cdd b) { return cdd{dd_dot2(a.x, b.x, -a.y, b.y), dd_dot2(a.x, b.y, a.y, b.x)}; }
__device__ __forceinline__ cdd cmul_nr(cdd a, cdd b) {
  return cdd{dd_dot2_nr(a.x, b.x, -a.y, b.y), dd_dot2_nr(a.x, b.y, a.y, b.x)};
}
__device__ __forceinline__ cdd operator+(cdd a, cdd b) { return cdd{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cdd operator-(cdd a, cdd b) { return cdd{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ cdd add_nr(cdd a, cdd b) { return cdd{add_nr(a.x, b.x), add_nr(a.y, b.y)}; }
__device__ __forceinline__ cdd sub_nr(cdd a, cdd b) { return cdd{add_nr(a.x, -b.x), add_nr(a.y, -b.y)}; }

// FP64 -> double-float with integer operations only: conversions between
// FP64 and FP32 run at the FP64 rate on GB300 (measured ~580 G/s against
// 38.9 T FFMA/s), which would cost as much as the transform itself.  hi takes
// the sign, exponent and top 23 fraction bits (truncated); lo is the
// remaining 29 fraction bits rounded to 24 and scaled by 2^(e-1075); then the
// pair is renormalised.  |v| below 2^-126 is flushed to zero (absolute error
// under 1.2e-38); Inf and NaN stay Inf and NaN.
__device__ __forceinline__ dd dd_from_double(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff);
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  if (e == 0x7ff) return dd(m ? __int_as_float(0x7fc00000) : __uint_as_float(sign | 0x7f800000u), 0.f);
  const int ef = e - 1023 + 127;
  if (ef < 1) return dd(__uint_as_float(sign), 0.f);
  if (ef > 254) return dd(__uint_as_float(sign | 0x7f800000u), 0.f);
  const float hi = __uint_as_float(sign | ((unsigned)ef << 23) | (unsigned)(m >> 29));
  const unsigned r = (unsigned)(m & 0x1FFFFFFFull);
  float lo = 0.f;
  if (r) {
    const unsigned fb = __float_as_uint(__uint2float_rn(r));  // exact to 24 bits, exponent field <= 127+28
    const int elo = (int)((fb >> 23) & 0xff) + (e - 1075);
    if (elo >= 1) lo = __uint_as_float(sign | ((unsigned)elo << 23) | (fb & 0x7fffffu));
  }
  return fast_two_sum(hi, lo);
}
__device__ __forceinline__ double dd_to_double(dd a) { return (double)a.hi + (double)a.lo; }

// FP32 -> FP64 by bit assembly (sign, exponent rebiased by 1023-127, fraction
// shifted into place): exact for normal numbers, zero for FP32 subnormals
// (below 1.2e-38), Inf/NaN kept.  Integer operations only, where the
// conversion instruction would run on the FP64 pipe.
__device__ __forceinline__ double f32_to_f64_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long frac = (unsigned long long)(u & 0x7fffffu) << 29;
  if (e == 0u) return __longlong_as_double((long long)sign);
  const unsigned long long ef = (e == 0xffu) ? 0x7ffull : (unsigned long long)(e + 896u);
  return __longlong_as_double((long long)(sign | (ef << 52) | frac));
}
// double-float -> FP64 with one FP64 addition
__device__ __forceinline__ double dd_to_double_int(dd a) { return f32_to_f64_bits(a.hi) + f32_to_f64_bits(a.lo); }

// Conversions and constants per arithmetic type T (double, float, dd).
template <typename T> struct Num;
template <> struct Num<double> {
  __device__ static double from_double(double v) { return v; }
  __device__ static double to_double(double v) { return v; }
  __device__ static double abs(double v) { return fabs(v); }
  __device__ static double max(double a, double b) { return fmax(a, b); }
  __device__ static bool finite(double v) { return isfinite(v); }
  __device__ static constexpr double sqrt3_2() { return 0.86602540378443864676372317075294; }
  __device__ static constexpr double cos_pi8() { return 0.9238795325112867; }
  __device__ static constexpr double sin_pi8() { return 0.3826834323650898; }
  __device__ static constexpr double sqrt1_2() { return 0.7071067811865476; }
  __device__ static constexpr double cos_pi12() { return 0.9659258262890683; }
  __device__ static constexpr double sin_pi12() { return 0.25881904510252074; }
};
template <> struct Num<float> {
  __device__ static float from_double(double v) { return (float)v; }
  __device__ static double to_double(float v) { return (double)v; }
  __device__ static float abs(float v) { return fabsf(v); }
  __device__ static float max(float a, float b) { return fmaxf(a, b); }
  __device__ static bool finite(float v) { return isfinite(v); }
  __device__ static constexpr float sqrt3_2() { return 0.866025404f; }
  __device__ static constexpr float cos_pi8() { return 0.923879533f; }
  __device__ static constexpr float sin_pi8() { return 0.382683432f; }
  __device__ static constexpr float sqrt1_2() { return 0.707106781f; }
  __device__ static constexpr float cos_pi12() { return 0.965925826f; }
  __device__ static constexpr float sin_pi12() { return 0.258819045f; }
};
template <> struct Num<dd> {
  __device__ static dd from_double(double v) { return dd_from_double(v); }
  __device__ static double to_double(dd v) { return dd_to_double(v); }
  __device__ static dd abs(dd v) { return dd_abs(v); }
  __device__ static dd max(dd a, dd b) { return dd_max(a, b); }
  __device__ static bool finite(dd v) { return dd_isfinite(v); }
  __device__ static constexpr dd sqrt3_2() { return dd(0.866025388f, 1.55436251e-08f); }
  __device__ static constexpr dd cos_pi8() { return dd(0.923879504f, 2.83074897e-08f); }
  __device__ static constexpr dd sin_pi8() { return dd(0.382683426f, 6.22335072e-09f); }
  __device__ static constexpr dd sqrt1_2() { return dd(0.707106769f, 1.21016175e-08f); }
  __device__ static constexpr dd cos_pi12() { return dd(0.965925813f, 1.35678162e-08f); }
  __device__ static constexpr dd sin_pi12() { return dd(0.258819044f, 1.46619872e-09f); }
};

}  // namespace chgpu
