// Two independent float-float numbers side by side: lane x and lane y of float2 registers,
// operated on with the paired FP32 instructions of sm_100-class GPUs (__fadd2_rn, __fmul2_rn,
// __ffma2_rn: one instruction performs the same IEEE round-to-nearest operation on both
// lanes).  Every operation below is the df64.cuh algorithm of the same name applied to each
// lane, so lane x of a result equals, bit for bit, what the scalar f2 operation returns for
// the lane-x operands (and likewise for y), in half the FP32 instructions.
//
// Used where the WENO face flux evaluates the same formula twice on different data: the two
// Lax-Friedrichs sides of every reconstruction (the minus side's stencil reversed, which turns
// its formula into the plus side's).
#pragma once

#include <cuda_runtime.h>

#include "df64.cuh"

namespace gbmv {

__device__ __forceinline__ float2 v2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

struct f2v {
  float2 hi, lo;
  __device__ __forceinline__ f2v() : hi(make_float2(0.f, 0.f)), lo(make_float2(0.f, 0.f)) {}
  __device__ __forceinline__ f2v(float2 h, float2 l) : hi(h), lo(l) {}
  // lane x = a, lane y = b
  __device__ __forceinline__ f2v(f2 a, f2 b) : hi(make_float2(a.hi, b.hi)), lo(make_float2(a.lo, b.lo)) {}
  // the same value in both lanes
  __device__ __forceinline__ explicit f2v(f2 a) : hi(v2(a.hi)), lo(v2(a.lo)) {}
  __device__ __forceinline__ f2 x() const { return f2(hi.x, lo.x); }
  __device__ __forceinline__ f2 y() const { return f2(hi.y, lo.y); }
  __device__ __forceinline__ float2 to_float() const { return add2(hi, lo); }
};

__device__ __forceinline__ f2v quick_two_sum2(float2 a, float2 b) {  // |a| >= |b| per lane
  const float2 s = add2(a, b);
  return f2v(s, sub2(b, sub2(s, a)));
}

__device__ __forceinline__ f2v two_sum2(float2 a, float2 b) {
  const float2 s = add2(a, b);
  const float2 bb = sub2(s, a);
  return f2v(s, add2(sub2(a, sub2(s, bb)), sub2(b, bb)));
}

__device__ __forceinline__ f2v two_prod2(float2 a, float2 b) {
  const float2 p = mul2(a, b);
  return f2v(p, fma2(a, b, neg2(p)));
}

__device__ __forceinline__ f2v operator+(f2v x, f2v y) {
  const f2v s = two_sum2(x.hi, y.hi);
  const float2 e = add2(s.lo, add2(x.lo, y.lo));
  return quick_two_sum2(s.hi, e);
}
__device__ __forceinline__ f2v operator-(f2v x) { return f2v(neg2(x.hi), neg2(x.lo)); }
__device__ __forceinline__ f2v operator-(f2v x, f2v y) { return x + (-y); }

__device__ __forceinline__ f2v operator*(f2v x, f2v y) {
  const f2v p = two_prod2(x.hi, y.hi);
  const float2 e = fma2(x.hi, y.lo, fma2(x.lo, y.hi, p.lo));
  return quick_two_sum2(p.hi, e);
}

// as f2 operator/: approximate reciprocal (one per lane), q1, remainder in float-float, q2
__device__ __forceinline__ f2v operator/(f2v x, f2v y) {
  const float2 ry = make_float2(__fdividef(1.f, y.hi.x), __fdividef(1.f, y.hi.y));
  const float2 q1 = mul2(x.hi, ry);
  const f2v r = x - y * f2v(q1, make_float2(0.f, 0.f));
  const float2 q2 = mul2(r.hi, ry);
  return quick_two_sum2(q1, q2);
}

// exact scaling by a power of two
__device__ __forceinline__ f2v f2v_scale(f2v x, float p2) {
  return f2v(mul2(x.hi, v2(p2)), mul2(x.lo, v2(p2)));
}

__device__ __forceinline__ f2v f2v_sqr(f2v x) {
  const f2v p = two_prod2(x.hi, x.hi);
  const float2 e = fma2(mul2(v2(2.f), x.hi), x.lo, p.lo);
  return quick_two_sum2(p.hi, e);
}

// per-lane minimum in the f2 order (hi first, then lo)
__device__ __forceinline__ f2v f2v_min(f2v a, f2v b) {
  const bool bx = b.hi.x < a.hi.x || (b.hi.x == a.hi.x && b.lo.x < a.lo.x);
  const bool by = b.hi.y < a.hi.y || (b.hi.y == a.hi.y && b.lo.y < a.lo.y);
  return f2v(make_float2(bx ? b.hi.x : a.hi.x, by ? b.hi.y : a.hi.y),
             make_float2(bx ? b.lo.x : a.lo.x, by ? b.lo.y : a.lo.y));
}

}  // namespace gbmv
