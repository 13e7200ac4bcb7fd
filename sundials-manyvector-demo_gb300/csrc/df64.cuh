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
  __host__ __device__ constexpr f2(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
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

__device__ __forceinline__ f2 operator/(f2 x, f2 y) {
  const float q1 = x.hi / y.hi;
  const f2 r = x - y * f2(q1, 0.f);
  const float q2 = r.hi / y.hi;
  return quick_two_sum(q1, q2);
}

}  // namespace gbmv
