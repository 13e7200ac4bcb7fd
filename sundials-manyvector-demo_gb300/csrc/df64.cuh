// Float-float ("double-single") arithmetic on the FP32 pipes: a value is hi + lo with
// |lo| <= ulp(hi)/2, about 48 significant bits.  Algorithms: Dekker's error-free
// transformations (Dekker 1971, "A floating-point technique for extending the available
// precision"; Knuth's TwoSum) as arranged in Bailey/Hida/Li's double-double library, with the
// FMA-based exact product.  GB300 retires FP32 FMAs 64x faster than FP64 ones, so this is how
// the mixed-precision WENO form keeps FP64-class precision in its smoothness indicators and
// nonlinear weights without paying for the FP64 pipe.
#pragma once

#include <cuda_runtime.h>

namespace gbmv {

struct f2 {
  float hi, lo;
  __host__ __device__ constexpr f2() : hi(0.f), lo(0.f) {}
  __host__ __device__ constexpr f2(float h, float l) : hi(h), lo(l) {}
  // from a double constant (split into the nearest float and the rounded remainder)
  __host__ __device__ constexpr explicit f2(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ constexpr explicit f2(int i) : hi((float)i), lo(0.f) {}
  __device__ __forceinline__ static f2 from(float x) { return f2(x, 0.f); }
  __device__ __forceinline__ float to_float() const { return hi + lo; }
  __device__ __forceinline__ double to_double() const { return (double)hi + (double)lo; }
};

__device__ __forceinline__ f2 quick_two_sum(float a, float b) {  // requires |a| >= |b|
  const float s = a + b;
  return f2(s, b - (s - a));
}

__device__ __forceinline__ f2 two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return f2(s, (a - (s - bb)) + (b - bb));
}

__device__ __forceinline__ f2 two_prod(float a, float b) {
  const float p = a * b;
  return f2(p, fmaf(a, b, -p));
}

__device__ __forceinline__ f2 operator+(f2 x, f2 y) {
  f2 s = two_sum(x.hi, y.hi);
  const float e = s.lo + (x.lo + y.lo);
  return quick_two_sum(s.hi, e);
}
__device__ __forceinline__ f2 operator-(f2 x) { return f2(-x.hi, -x.lo); }
__device__ __forceinline__ f2 operator-(f2 x, f2 y) { return x + (-y); }

__device__ __forceinline__ f2 operator*(f2 x, f2 y) {
  f2 p = two_prod(x.hi, y.hi);
  const float e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, p.lo));
  return quick_two_sum(p.hi, e);
}

// Division: q1 from a fast approximate reciprocal, the remainder x - y*q1 formed in
// float-float, one correction q2 -- the correction absorbs q1's few-ulp error, so the result
// keeps the float-float precision.
__device__ __forceinline__ f2 operator/(f2 x, f2 y) {
  const float ry = __fdividef(1.f, y.hi);
  const float q1 = x.hi * ry;
  const f2 r = x - y * f2(q1, 0.f);
  const float q2 = r.hi * ry;
  return quick_two_sum(q1, q2);
}

// exact scaling by a power of two
__device__ __forceinline__ f2 f2_scale(f2 x, float p2) { return f2(x.hi * p2, x.lo * p2); }

// x^2 with the exact square of the high part
__device__ __forceinline__ f2 f2_sqr(f2 x) {
  f2 p = two_prod(x.hi, x.hi);
  const float e = fmaf(2.f * x.hi, x.lo, p.lo);
  return quick_two_sum(p.hi, e);
}

// exact split of a double into hi + lo (48 of its 53 significant bits survive)
__device__ __forceinline__ f2 f2_from_double(double d) {
  const float h = __double2float_rn(d);
  return f2(h, __double2float_rn(d - (double)h));
}

// Conversions between double and float from the bit patterns, with integer instructions.
// Conversion instructions with a 64-bit operand run at the FP64 rate, 1/64 of the FP32 rate on
// GB300, so in passes that mostly convert (the float-float primitives, the FP32 factors of the
// Newton matrices) they set the time.  Each helper returns exactly what the round-to-nearest
// hardware conversion returns: the integer path covers every normal float result, anything
// else (zero, subnormal, overflow, inf, NaN) takes the hardware conversion.

// double -> float, round to nearest even: drop 29 mantissa bits on the pattern (a carry into
// the exponent is the correct rounding), re-bias the exponent (1023 - 127 = 896)
__device__ __forceinline__ float f32_of_f64(double d) {
  const unsigned long long p = (unsigned long long)__double_as_longlong(d);
  const unsigned e = (unsigned)(p >> 52) & 0x7FFu;
  if (e - 897u > 1149u - 897u) return __double2float_rn(d);  // result not surely a normal float
  const unsigned long long r = p + 0x0FFFFFFFull + ((p >> 29) & 1ull);
  const unsigned hi = (unsigned)(r >> 32);
  const unsigned s = hi & 0x80000000u;
  const unsigned er = (hi >> 20) & 0x7FFu;
  const unsigned m = (unsigned)(r >> 29) & 0x7FFFFFu;
  return __uint_as_float(s | ((er - 896u) << 23) | m);
}

// float -> double, exact
__device__ __forceinline__ double f64_of_f32(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  if (e - 1u > 253u) return (double)f;  // zero, subnormal, inf, NaN
  const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3);
  const unsigned lo = u << 29;
  return __hiloint2double((int)hi, (int)lo);
}

// f2_from_double without conversion instructions (bit-identical to it)
__device__ __forceinline__ f2 f2_split(double d) {
  const float h = f32_of_f64(d);
  return f2(h, f32_of_f64(d - f64_of_f32(h)));
}

// f2::to_double without conversion instructions (bit-identical to it)
__device__ __forceinline__ double f2_to_double(f2 x) {
  return f64_of_f32(x.hi) + f64_of_f32(x.lo);
}

__device__ __forceinline__ bool operator<(f2 a, f2 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(f2 a, f2 b) { return b < a; }
__device__ __forceinline__ bool operator<=(f2 a, f2 b) { return !(b < a); }
__device__ __forceinline__ bool operator==(f2 a, f2 b) { return a.hi == b.hi && a.lo == b.lo; }
__device__ __forceinline__ f2 f2_fabs(f2 a) { return a.hi < 0.f ? -a : a; }
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) { return a * b + c; }

// square root: FP32 estimate, one Newton correction in float-float
__device__ __forceinline__ f2 f2_sqrt(f2 a) {
  if (!(a.hi > 0.f)) return f2(0.f, 0.f);
  const float s = sqrtf(a.hi);
  const f2 ss = two_prod(s, s);
  const float r = ((a.hi - ss.hi) - ss.lo + a.lo) / (2.f * s);
  return quick_two_sum(s, r);
}

}  // namespace gbmv
