// WENO5 characteristic face flux (the reference's face_flux, src/utilities.cpp:270-479),
// written once for two arithmetic types:
//   T = double : the FP64 form (parity with the reference to rounding);
//   T = f2     : float-float arithmetic (~48-bit significand) on the FP32 pipes -- the
//                mixed-precision form.  GB300 retires FP32 FMAs 64x faster than FP64 ones, and
//                the reference's eigenvector basis (built with c^2 where c is expected,
//                src/utilities.cpp:309) is ill-conditioned when c is small in code units, so
//                plain FP32 characteristic arithmetic loses too many digits; float-float keeps
//                FP64-class accuracy.  Any split flux beyond 1e18 in magnitude (where the
//                float exponent range would overflow a square) falls back to native FP64.
//
// Arrangement (both types), chosen to spend few instructions on the slow pipe:
//   * nonlinear weights normalised by the smallest a_k = eps + beta_k (no overflow) and one
//     final division -- for doubles the equivalent product form with ONE division;
//   * Lax-Friedrichs splitting folded into one FMA per value (0.5 f +- (0.5 alpha) w); tracers
//     one multiply (c_j * 0.5 (u_j +- alpha));
//   * the sparse rows of the eigenvector matrices applied without their zeros.
// Results agree with the reference's to a few ulps of each face flux (FP64 form).
#pragma once

#include "common.cuh"
#include "df64.cuh"
#include "df64x2.cuh"

namespace gbmv {

// ---- conversions used by the type-generic code
__device__ __forceinline__ double num_from(double d, double*) { return d; }
__device__ __forceinline__ f2 num_from(double d, f2*) { return f2_from_double(d); }

__device__ __forceinline__ double num_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ f2 num_sqrt(f2 x) { return f2_sqrt(x); }
__device__ __forceinline__ double num_fabs(double x) { return fabs(x); }
__device__ __forceinline__ f2 num_fabs(f2 x) { return f2_fabs(x); }
__device__ __forceinline__ double num_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ f2 num_fma(f2 a, f2 b, f2 c) { return f2_fma(a, b, c); }

template <typename T>
__device__ __forceinline__ T sqrt0(T x) {
  return x <= T(0.0) ? T(0.0) : num_sqrt(x);
}

__device__ __forceinline__ double eos64(double gamma, double rho, double mx, double my, double mz,
                                        double et) {
  return (gamma - 1.0) * (et - (mx * mx + my * my + mz * mz) * 0.5 / rho);
}

template <typename T>
__device__ __forceinline__ T eos_t(T gm, T rho, T mx, T my, T mz, T et) {
  return gm * (et - (mx * mx + my * my + mz * mz) * T(0.5) / rho);
}

// Smoothness indicators of the three candidate stencils of f0..f4 (Jiang-Shu, as the
// reference: beta = 13/12 (second difference)^2 + 1/4 (first-difference combination)^2).
template <typename T>
__device__ __forceinline__ void weno_betas(T f0, T f1, T f2_, T f3, T f4, T& bA, T& bB, T& bC) {
  const T b13 = T(13.0 / 12.0), q = T(0.25);
  const T dA = f2_ - T(2.0) * f3 + f4, eA = T(3.0) * f2_ - T(4.0) * f3 + f4;
  const T dB = f1 - T(2.0) * f2_ + f3, eB = f1 - f3;
  const T dC = f0 - T(2.0) * f1 + f2_, eC = f0 - T(4.0) * f1 + T(3.0) * f2_;
  bA = b13 * (dA * dA) + q * (eA * eA);
  bB = b13 * (dB * dB) + q * (eB * eB);
  bC = b13 * (dC * dC) + q * (eC * eC);
}

// sum_k q_k d_k / a_k^2 / sum_k d_k / a_k^2 with a_k = eps + beta_k.
__device__ __forceinline__ double weno_combine(double bA, double bB, double bC, double qA,
                                               double qB, double qC, double dA, double dB,
                                               double dC) {
  // product form, one division: weights d_k * prod_{j != k} a_j^2 (a_k >= 1e-6)
  const double eps = 1e-6;
  double aA = eps + bA, aB = eps + bB, aC = eps + bC;
  aA = aA * aA;
  aB = aB * aB;
  aC = aC * aC;
  const double tA = dA * (aB * aC), tB = dB * (aA * aC), tC = dC * (aA * aB);
  return (tA * qA + tB * qB + tC * qC) / (tA + tB + tC);
}

// Upwind-biased reconstruction at x_{i+1/2} from f0..f4 = points i-2..i+2 (linear weights
// 0.3, 0.6, 0.1 for candidates {f2,f3,f4}, {f1,f2,f3}, {f0,f1,f2}); mirror image for the
// left-moving part from points i-1..i+3.
template <bool Plus, typename T>
__device__ __forceinline__ T weno_side(T f0, T f1, T f2_, T f3, T f4) {
  T bA, bB, bC;
  weno_betas(f0, f1, f2_, f3, f4, bA, bB, bC);
  const T c13 = T(1.0 / 3.0), c56 = T(5.0 / 6.0), c16 = T(1.0 / 6.0), c76 = T(7.0 / 6.0),
          c116 = T(11.0 / 6.0);
  if (Plus) {
    const T qA = c13 * f2_ + c56 * f3 - c16 * f4;
    const T qB = -c16 * f1 + c56 * f2_ + c13 * f3;
    const T qC = c13 * f0 - c76 * f1 + c116 * f2_;
    return weno_combine(bA, bB, bC, qA, qB, qC, T(0.3), T(0.6), T(0.1));
  } else {
    const T qA = c116 * f2_ - c76 * f3 + c13 * f4;
    const T qB = c13 * f1 + c56 * f2_ - c16 * f3;
    const T qC = -c16 * f0 + c56 * f1 + c13 * f2_;
    return weno_combine(bA, bB, bC, qA, qB, qC, T(0.1), T(0.6), T(0.3));
  }
}

template <bool Plus>
__device__ __forceinline__ double weno_safe(double f0, double f1, double f2_, double f3, double f4) {
  return weno_side<Plus>(f0, f1, f2_, f3, f4);
}
// float-float with a native-FP64 fallback for values whose squares would leave the float
// range.  Kept out of line: one copy of the long float-float sequence serves all 2*NVAR
// reconstructions of a face, which keeps the kernel inside the instruction cache.
// Float-float reconstruction arranged for fewer float-float operations than the reference's
// literal formula (same mathematics, ~48-bit arithmetic):
//   * the four neighbour differences D01..D34 serve all six indicator terms and all three
//     candidate polynomials;
//   * the weights are d_k (a_min / a_k)^2 with a_k = eps + beta_k, ratios in (0, 1], so
//     nothing leaves the float exponent range.
template <bool Plus>
__device__ __noinline__ f2 weno_side_f2(f2 f0, f2 f1, f2 f2_, f2 f3, f2 f4) {
  const f2 D01 = f0 - f1, D12 = f1 - f2_, D23 = f2_ - f3, D34 = f3 - f4;
  const f2 dA = D23 - D34, dB = D12 - D23, dC = D01 - D12;       // second differences
  const f2 eA = dA + f2_scale(D23, 2.f), eB = D12 + D23, eC = dC - f2_scale(D12, 2.f);
  const f2 b13(13.0 / 12.0), sixth(1.0 / 6.0), eps(1e-6);
  f2 aA = eps + (b13 * f2_sqr(dA) + f2_scale(f2_sqr(eA), 0.25f));
  f2 aB = eps + (b13 * f2_sqr(dB) + f2_scale(f2_sqr(eB), 0.25f));
  f2 aC = eps + (b13 * f2_sqr(dC) + f2_scale(f2_sqr(eC), 0.25f));
  // candidates: (2f2+5f3-f4)/6 etc. written around their central value
  f2 qA, qB, qC, wA, wB, wC;
  if (Plus) {
    qA = f3 + sixth * (f2_scale(D23, 2.f) + D34);
    qB = f2_ - sixth * (D12 + f2_scale(D23, 2.f));
    qC = f2_ + sixth * (f2_scale(D01, 2.f) - f2(5.0) * D12);
    wA = f2(0.3); wB = f2(0.6); wC = f2(0.1);
  } else {
    qA = f2_ + sixth * (f2(5.0) * D23 - f2_scale(D34, 2.f));
    qB = f2_ + sixth * (f2_scale(D12, 2.f) + D23);
    qC = f1 - sixth * (D01 + f2_scale(D12, 2.f));
    wA = f2(0.1); wB = f2(0.6); wC = f2(0.3);
  }
  // weights relative to the smallest a: ratios in (0, 1], nothing leaves the float range
  f2 m = aA < aB ? aA : aB;
  m = m < aC ? m : aC;
  const f2 rA = m / aA, rB = m / aB, rC = m / aC;
  const f2 tA = wA * f2_sqr(rA), tB = wB * f2_sqr(rB), tC = wC * f2_sqr(rC);
  return (tA * qA + tB * qB + tC * qC) / (tA + tB + tC);
}
template <bool Plus>
__device__ __noinline__ f2 weno_side_f2_fallback(f2 f0, f2 f1, f2 f2_, f2 f3, f2 f4) {
  const double r = weno_side<Plus>(f0.to_double(), f1.to_double(), f2_.to_double(),
                                   f3.to_double(), f4.to_double());
  return f2_from_double(r);
}
template <bool Plus>
__device__ __forceinline__ f2 weno_safe(f2 f0, f2 f1, f2 f2_, f2 f3, f2 f4) {
  const float m = fmaxf(fmaxf(fmaxf(fabsf(f0.hi), fabsf(f1.hi)), fmaxf(fabsf(f2_.hi), fabsf(f3.hi))),
                        fabsf(f4.hi));
  if (m < 1e18f) return weno_side_f2<Plus>(f0, f1, f2_, f3, f4);
  return weno_side_f2_fallback<Plus>(f0, f1, f2_, f3, f4);
}

// Reconstruction in correction form (GBMV_MIXED_FAST, species fields): with the central point f2_
// in float-float, r = f2_ + sum_k w_k (q_k - f2_).  The corrections q_k - f2_ and the
// smoothness indicators are built from the neighbour differences D01..D34 (exact float-float
// subtractions, then rounded to float), and the weights and the weighted correction are FP32:
// a relative weight error e changes r by e |q_k - f2_| -- an O(dx) difference in smooth flow,
// the jump across a discontinuity -- never by e |r|, because the base value is not weighted
// (the three weights need not sum to exactly one).  Used for the componentwise species
// reconstructions only: the characteristic values of the fluid part are back-projected through
// an eigenbasis with condition ~1/c^2, which would amplify the weight rounding (measured:
// 2e-5 on the chem-hydro state).
template <bool Plus>
__device__ __noinline__ f2 weno_side_f2d(f2 f0, f2 f1, f2 f2_, f2 f3, f2 f4) {
  const float D01 = (f0 - f1).to_float(), D12 = (f1 - f2_).to_float(),
              D23 = (f2_ - f3).to_float(), D34 = (f3 - f4).to_float();
  const float dA = D23 - D34, dB = D12 - D23, dC = D01 - D12;  // second differences
  const float eA = dA + 2.f * D23, eB = D12 + D23, eC = dC - 2.f * D12;
  const float b13 = 13.f / 12.f, sixth = 1.f / 6.f;
  const float aA = 1e-6f + (b13 * (dA * dA) + 0.25f * (eA * eA));
  const float aB = 1e-6f + (b13 * (dB * dB) + 0.25f * (eB * eB));
  const float aC = 1e-6f + (b13 * (dC * dC) + 0.25f * (eC * eC));
  float cA, cB, cC, wA, wB, wC;  // candidate minus central point, linear weights
  if (Plus) {
    cA = (D34 - 4.f * D23) * sixth;
    cB = -(D12 + 2.f * D23) * sixth;
    cC = (2.f * D01 - 5.f * D12) * sixth;
    wA = 0.3f; wB = 0.6f; wC = 0.1f;
  } else {
    cA = (5.f * D23 - 2.f * D34) * sixth;
    cB = (2.f * D12 + D23) * sixth;
    cC = (4.f * D12 - D01) * sixth;
    wA = 0.1f; wB = 0.6f; wC = 0.3f;
  }
  const float m = fminf(fminf(aA, aB), aC);
  const float rA = m / aA, rB = m / aB, rC = m / aC;
  const float tA = wA * (rA * rA), tB = wB * (rB * rB), tC = wC * (rC * rC);
  const float corr = (tA * cA + tB * cB + tC * cC) / (tA + tB + tC);
  return f2_ + f2(corr, 0.f);
}
template <bool Plus>
__device__ __forceinline__ f2 weno_safe_d(f2 f0, f2 f1, f2 f2_, f2 f3, f2 f4) {
  const float m = fmaxf(fmaxf(fmaxf(fabsf(f0.hi), fabsf(f1.hi)), fmaxf(fabsf(f2_.hi), fabsf(f3.hi))),
                        fabsf(f4.hi));
  if (m < 1e18f) return weno_side_f2d<Plus>(f0, f1, f2_, f3, f4);
  return weno_side_f2_fallback<Plus>(f0, f1, f2_, f3, f4);
}
template <bool Plus>
__device__ __forceinline__ double weno_safe_d(double f0, double f1, double f2_, double f3,
                                              double f4) {
  return weno_safe<Plus>(f0, f1, f2_, f3, f4);
}
// WV = 0: weights in the arithmetic type T; WV = 1: the correction form above
template <bool Plus, int WV, typename T>
__device__ __forceinline__ T weno_pick(T f0, T f1, T f2_, T f3, T f4) {
  if constexpr (WV == 1) return weno_safe_d<Plus>(f0, f1, f2_, f3, f4);
  else return weno_safe<Plus>(f0, f1, f2_, f3, f4);
}

// Paired reconstructions (df64x2.cuh): both Lax-Friedrichs sides of a face in one pass, lane x
// the plus side from f0..f4, lane y the minus side with its stencil reversed -- the minus
// formula on g0..g4 is the plus formula on g4..g0 (the candidates, linear weights and
// smoothness indicators map onto each other under the reversal) -- so one instruction stream
// serves both.  Lane x returns exactly weno_side_f2<true>'s value; lane y the minus side's
// value up to the rounding of the mirrored evaluation order.
__device__ __forceinline__ f2v weno_plus_f2v_body(f2v f0, f2v f1, f2v f2_, f2v f3, f2v f4) {
  const f2v D01 = f0 - f1, D12 = f1 - f2_, D23 = f2_ - f3, D34 = f3 - f4;
  const f2v dA = D23 - D34, dB = D12 - D23, dC = D01 - D12;  // second differences
  const f2v eA = dA + f2v_scale(D23, 2.f), eB = D12 + D23, eC = dC - f2v_scale(D12, 2.f);
  const f2v b13(f2(13.0 / 12.0)), sixth(f2(1.0 / 6.0)), eps(f2(1e-6));
  const f2v aA = eps + (b13 * f2v_sqr(dA) + f2v_scale(f2v_sqr(eA), 0.25f));
  const f2v aB = eps + (b13 * f2v_sqr(dB) + f2v_scale(f2v_sqr(eB), 0.25f));
  const f2v aC = eps + (b13 * f2v_sqr(dC) + f2v_scale(f2v_sqr(eC), 0.25f));
  const f2v qA = f3 + sixth * (f2v_scale(D23, 2.f) + D34);
  const f2v qB = f2_ - sixth * (D12 + f2v_scale(D23, 2.f));
  const f2v qC = f2_ + sixth * (f2v_scale(D01, 2.f) - f2v(f2(5.0)) * D12);
  const f2v m = f2v_min(f2v_min(aA, aB), aC);
  const f2v rA = m / aA, rB = m / aB, rC = m / aC;
  const f2v tA = f2v(f2(0.3)) * f2v_sqr(rA), tB = f2v(f2(0.6)) * f2v_sqr(rB),
            tC = f2v(f2(0.1)) * f2v_sqr(rC);
  return (tA * qA + tB * qB + tC * qC) / (tA + tB + tC);
}
// the correction form of weno_side_f2d (species fields of GBMV_MIXED_FAST), paired
__device__ __forceinline__ f2v weno_plus_f2dv_body(f2v f0, f2v f1, f2v f2_, f2v f3, f2v f4) {
  const float2 D01 = (f0 - f1).to_float(), D12 = (f1 - f2_).to_float(),
               D23 = (f2_ - f3).to_float(), D34 = (f3 - f4).to_float();
  const float2 dA = sub2(D23, D34), dB = sub2(D12, D23), dC = sub2(D01, D12);
  const float2 eA = fma2(v2(2.f), D23, dA), eB = add2(D12, D23), eC = fma2(v2(-2.f), D12, dC);
  const float2 b13 = v2(13.f / 12.f), q = v2(0.25f), sixth = v2(1.f / 6.f);
  const float2 aA = add2(v2(1e-6f), fma2(b13, mul2(dA, dA), mul2(q, mul2(eA, eA))));
  const float2 aB = add2(v2(1e-6f), fma2(b13, mul2(dB, dB), mul2(q, mul2(eB, eB))));
  const float2 aC = add2(v2(1e-6f), fma2(b13, mul2(dC, dC), mul2(q, mul2(eC, eC))));
  // candidate minus central point (plus side: linear weights 0.3, 0.6, 0.1)
  const float2 cA = mul2(fma2(v2(-4.f), D23, D34), sixth);
  const float2 cB = mul2(fma2(v2(2.f), D23, D12), v2(-1.f / 6.f));
  const float2 cC = mul2(fma2(v2(-5.f), D12, mul2(v2(2.f), D01)), sixth);
  const float2 m = make_float2(fminf(fminf(aA.x, aB.x), aC.x), fminf(fminf(aA.y, aB.y), aC.y));
  // ratios in (0, 1] and a sum of weights above 0.1: the fast reciprocal is accurate here
  const float2 rA = make_float2(__fdividef(m.x, aA.x), __fdividef(m.y, aA.y));
  const float2 rB = make_float2(__fdividef(m.x, aB.x), __fdividef(m.y, aB.y));
  const float2 rC = make_float2(__fdividef(m.x, aC.x), __fdividef(m.y, aC.y));
  const float2 tA = mul2(v2(0.3f), mul2(rA, rA)), tB = mul2(v2(0.6f), mul2(rB, rB)),
               tC = mul2(v2(0.1f), mul2(rC, rC));
  const float2 num = fma2(tA, cA, fma2(tB, cB, mul2(tC, cC)));
  const float2 den = add2(add2(tA, tB), tC);
  const float2 corr = make_float2(__fdividef(num.x, den.x), __fdividef(num.y, den.y));
  return f2_ + f2v(corr, make_float2(0.f, 0.f));
}
// One out-of-line copy of each serves every reconstruction of a face (the kernel stays inside
// the instruction cache); the x2 forms take two independent reconstructions at once, two
// dependency chains the scheduler interleaves.
static __device__ __noinline__ f2v weno_plus_f2v(f2v f0, f2v f1, f2v f2_, f2v f3, f2v f4) {
  return weno_plus_f2v_body(f0, f1, f2_, f3, f4);
}
static __device__ __noinline__ f2v weno_plus_f2dv(f2v f0, f2v f1, f2v f2_, f2v f3, f2v f4) {
  return weno_plus_f2dv_body(f0, f1, f2_, f3, f4);
}
struct f2v2 {
  f2v a, b;
};
template <int WV>
static __device__ __noinline__ f2v2 weno_plus_x2(f2v a0, f2v a1, f2v a2, f2v a3, f2v a4,
                                                 f2v b0, f2v b1, f2v b2, f2v b3, f2v b4) {
  f2v2 r;
  if constexpr (WV == 1) {
    r.a = weno_plus_f2dv_body(a0, a1, a2, a3, a4);
    r.b = weno_plus_f2dv_body(b0, b1, b2, b3, b4);
  } else {
    r.a = weno_plus_f2v_body(a0, a1, a2, a3, a4);
    r.b = weno_plus_f2v_body(b0, b1, b2, b3, b4);
  }
  return r;
}

// both sides of a face: lane x the plus side from f0..f4, lane y the minus side whose stencil
// g0..g4 is held reversed (f0.y = g4, ..., f4.y = g0); values beyond 1e18 in magnitude (where
// float squares would overflow) go to the per-side FP64 fallback
template <int WV>
__device__ __forceinline__ f2v weno_pair(f2v f0, f2v f1, f2v f2_, f2v f3, f2v f4) {
  float mx = 0.f;
  mx = fmaxf(mx, fmaxf(fabsf(f0.hi.x), fabsf(f0.hi.y)));
  mx = fmaxf(mx, fmaxf(fabsf(f1.hi.x), fabsf(f1.hi.y)));
  mx = fmaxf(mx, fmaxf(fabsf(f2_.hi.x), fabsf(f2_.hi.y)));
  mx = fmaxf(mx, fmaxf(fabsf(f3.hi.x), fabsf(f3.hi.y)));
  mx = fmaxf(mx, fmaxf(fabsf(f4.hi.x), fabsf(f4.hi.y)));
  if (mx < 1e18f) {
    if constexpr (WV == 1) return weno_plus_f2dv(f0, f1, f2_, f3, f4);
    else return weno_plus_f2v(f0, f1, f2_, f3, f4);
  }
  const f2 rx = weno_side_f2_fallback<true>(f0.x(), f1.x(), f2_.x(), f3.x(), f4.x());
  const f2 ry = weno_side_f2_fallback<false>(f4.y(), f3.y(), f2_.y(), f1.y(), f0.y());
  return f2v(rx, ry);
}

__device__ __forceinline__ float f2v_absmax(f2v a) {
  return fmaxf(fabsf(a.hi.x), fabsf(a.hi.y));
}
template <int WV>
__device__ __forceinline__ f2v2 weno_pair_x2(f2v a0, f2v a1, f2v a2, f2v a3, f2v a4, f2v b0,
                                             f2v b1, f2v b2, f2v b3, f2v b4) {
  float mx = fmaxf(fmaxf(f2v_absmax(a0), f2v_absmax(a1)), fmaxf(f2v_absmax(a2), f2v_absmax(a3)));
  mx = fmaxf(mx, fmaxf(fmaxf(f2v_absmax(a4), f2v_absmax(b0)), fmaxf(f2v_absmax(b1), f2v_absmax(b2))));
  mx = fmaxf(mx, fmaxf(f2v_absmax(b3), f2v_absmax(b4)));
  if (mx < 1e18f) return weno_plus_x2<WV>(a0, a1, a2, a3, a4, b0, b1, b2, b3, b4);
  f2v2 r;
  r.a = weno_pair<WV>(a0, a1, a2, a3, a4);
  r.b = weno_pair<WV>(b0, b1, b2, b3, b4);
  return r;
}

// Face-local data shared by the fluid and tracer parts.
template <typename T>
struct FaceState {
  T hp[6], hm[6];  // 0.5 (u_j + alpha), 0.5 (u_j - alpha): tracer split-flux factors
};

// Fluid part: W[j] = (rho, m_normal, m_t1, m_t2, et) of stencil point j (after the direction
// swap); writes the five fluxes in the same order.
// Per-point primitives computed once per cell (pressure, normal velocity, sound speed).
template <typename T>
struct PointPrims {
  T p[6], u[6], c[6];
};

template <typename T, bool Pre = false, int WV = 0>
__device__ __forceinline__ void fluid_face_flux(const T (&W)[6][5], double gamma_d,
                                                FaceState<T>& S, T (&out)[5],
                                                const PointPrims<T>* pre = nullptr) {
  T* tag = nullptr;
  const T gamma = num_from(gamma_d, tag);
  const T gm = num_from(gamma_d - 1.0, tag);
  const T half(0.5), one(1.0);
  T p[6];
#pragma unroll
  for (int j = 0; j < 6; ++j)
    p[j] = Pre ? pre->p[j] : eos_t(gm, W[j][0], W[j][1], W[j][2], W[j][3], W[j][4]);
  // Roe average at the face (src/utilities.cpp:298-304)
  const T sL = sqrt0(W[2][0]), sR = sqrt0(W[3][0]);
  const T sbar = half * (sL + sR);
  T u, v, ww, H;
  if (Pre) {  // three divisions instead of twelve (float-float divisions are the costly op)
    const T isL = one / sL, isR = one / sR, hs = half / sbar;
    u = (W[2][1] * isL + W[3][1] * isR) * hs;
    v = (W[2][2] * isL + W[3][2] * isR) * hs;
    ww = (W[2][3] * isL + W[3][3] * isR) * hs;
    H = ((p[2] + W[2][4]) * isL + (p[3] + W[3][4]) * isR) * hs;
  } else {
    u = half * (W[2][1] / sL + W[3][1] / sR) / sbar;
    v = half * (W[2][2] / sL + W[3][2] / sR) / sbar;
    ww = half * (W[2][3] / sL + W[3][3] / sR) / sbar;
    H = half * ((p[2] + W[2][4]) / sL + (p[3] + W[3][4]) / sR) / sbar;
  }
  const T qsq = u * u + v * v + ww * ww;
  const T c = gm * (H - half * qsq);  // the reference's "csnd" (src/utilities.cpp:309)
  const T ci = one / c;
  // nonzero entries of the left eigenvector rows (src/utilities.cpp:342-364)
  const T hgc = half * gm * ci, hc = half * ci;
  const T L00 = hc * (u + half * gm * qsq), L01 = -hc * (gm * u + one), L02 = -v * hgc,
          L03 = -ww * hgc, L04 = hgc;
  const T gc = gm * ci;
  const T L30 = -gc * (qsq - H), L31 = u * gc, L32 = v * gc, L33 = ww * gc, L34 = -gc;
  const T L40 = -hc * (u - half * gm * qsq), L41 = -hc * (gm * u - one);

  // point fluxes (halved) and the Lax-Friedrichs speed (src/utilities.cpp:368-380)
  T hf[6][5];
  T alpha(0.0);
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const T uj = Pre ? pre->u[j] : W[j][1] / W[j][0];
    hf[j][0] = half * W[j][1];
    hf[j][1] = half * (uj * W[j][1] + p[j]);
    hf[j][2] = half * (uj * W[j][2]);
    hf[j][3] = half * (uj * W[j][3]);
    hf[j][4] = half * (uj * (W[j][4] + p[j]));
    S.hp[j] = uj;  // temporarily u_j
    const T s = num_fabs(uj) + (Pre ? pre->c[j] : sqrt0(gamma * p[j] / W[j][0]));
    alpha = (alpha < s) ? s : alpha;
  }
  const T ha = half * alpha;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const T uj = S.hp[j];
    S.hp[j] = half * uj + ha;
    S.hm[j] = half * uj - ha;
  }

  T ff[5];
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    T pr[5][5];  // projected split flux [point][characteristic component]
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const int pt = j + side;
      const T sa = side == 0 ? ha : -ha;
      T fs[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) fs[m] = num_fma(sa, W[pt][m], hf[pt][m]);
      pr[j][0] = L00 * fs[0] + L01 * fs[1] + L02 * fs[2] + L03 * fs[3] + L04 * fs[4];
      pr[j][1] = fs[2] - v * fs[0];
      pr[j][2] = fs[3] - ww * fs[0];
      pr[j][3] = L30 * fs[0] + L31 * fs[1] + L32 * fs[2] + L33 * fs[3] + L34 * fs[4];
      pr[j][4] = L40 * fs[0] + L41 * fs[1] + L02 * fs[2] + L03 * fs[3] + L04 * fs[4];
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      if (side == 0)
        ff[i] = weno_pick<true, WV>(pr[0][i], pr[1][i], pr[2][i], pr[3][i], pr[4][i]);
      else
        ff[i] = ff[i] + weno_pick<false, WV>(pr[0][i], pr[1][i], pr[2][i], pr[3][i], pr[4][i]);
    }
  }
  // right eigenvector columns (src/utilities.cpp:318-340)
  out[0] = ff[0] + ff[3] + ff[4];
  out[1] = (u - c) * ff[0] + u * ff[3] + (u + c) * ff[4];
  out[2] = v * ff[0] + ff[1] + v * ff[3] + v * ff[4];
  out[3] = ww * ff[0] + ff[2] + ww * ff[3] + ww * ff[4];
  out[4] = (H - u * c) * ff[0] + v * ff[1] + ww * ff[2] + (half * qsq) * ff[3] + (H + u * c) * ff[4];
}

// Tracer part for one advected field from its 6 stencil values.
template <typename T, int WV = 0>
__device__ __forceinline__ T tracer_face_flux(const FaceState<T>& S, const T (&cv)[6]) {
  T r = weno_pick<true, WV>(cv[0] * S.hp[0], cv[1] * S.hp[1], cv[2] * S.hp[2], cv[3] * S.hp[3],
                            cv[4] * S.hp[4]);
  r = r + weno_pick<false, WV>(cv[1] * S.hm[1], cv[2] * S.hm[2], cv[3] * S.hm[3],
                               cv[4] * S.hm[4], cv[5] * S.hm[5]);
  return r;
}

// Float-float fluid part with both Lax-Friedrichs sides paired (df64x2.cuh): the same
// arithmetic as fluid_face_flux<f2, true> up to the rounding of the mirrored minus side.
// Pair k holds side 0 at stencil point k in lane x and side 1 at point 5 - k in lane y, so the
// projected pairs feed weno_pair directly; the split fluxes are formed per pair from the point
// values (no per-point flux arrays are kept).
__device__ __forceinline__ void fluid_face_flux_f2v(const f2 (&W)[6][5], double gamma_d,
                                                    FaceState<f2>& S, f2 (&out)[5],
                                                    const PointPrims<f2>& pre) {
  const f2 gm = f2_from_double(gamma_d - 1.0);
  const f2 half(0.5), one(1.0);
  // Roe average at the face (src/utilities.cpp:298-304)
  const f2 sL = sqrt0(W[2][0]), sR = sqrt0(W[3][0]);
  const f2 sbar = half * (sL + sR);
  const f2 isL = one / sL, isR = one / sR, hs = half / sbar;
  const f2 u = (W[2][1] * isL + W[3][1] * isR) * hs;
  const f2 v = (W[2][2] * isL + W[3][2] * isR) * hs;
  const f2 ww = (W[2][3] * isL + W[3][3] * isR) * hs;
  const f2 H = ((pre.p[2] + W[2][4]) * isL + (pre.p[3] + W[3][4]) * isR) * hs;
  const f2 qsq = u * u + v * v + ww * ww;
  const f2 c = gm * (H - half * qsq);  // the reference's "csnd" (src/utilities.cpp:309)
  const f2 ci = one / c;
  // nonzero entries of the left eigenvector rows (src/utilities.cpp:342-364)
  const f2 hgc = half * gm * ci, hc = half * ci;
  const f2v L00(hc * (u + half * gm * qsq)), L01(-hc * (gm * u + one)), L02(-v * hgc),
      L03(-ww * hgc), L04(hgc);
  const f2 gc = gm * ci;
  const f2v L30(-gc * (qsq - H)), L31(u * gc), L32(v * gc), L33(ww * gc), L34(-gc);
  const f2v L40(-hc * (u - half * gm * qsq)), L41(-hc * (gm * u - one));
  const f2v vv(v), wv(ww);
  // Lax-Friedrichs speed (src/utilities.cpp:368-380)
  f2 alpha(0.0);
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const f2 s = f2_fabs(pre.u[j]) + pre.c[j];
    alpha = (alpha < s) ? s : alpha;
  }
  const f2 ha = half * alpha;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    S.hp[j] = half * pre.u[j] + ha;
    S.hm[j] = half * pre.u[j] - ha;
  }
  const f2v sa(ha, -ha);
  const f2v hv(half);
  f2v P[5][5];  // [pair][characteristic component]
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int a = k, b = 5 - k;
    const f2v uj(pre.u[a], pre.u[b]), pj(pre.p[a], pre.p[b]);
    f2v Wj[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) Wj[m] = f2v(W[a][m], W[b][m]);
    // halved point flux plus (or minus) 0.5 alpha w, as fluid_face_flux forms it
    f2v fs[5];
    fs[0] = sa * Wj[0] + hv * Wj[1];
    fs[1] = sa * Wj[1] + hv * (uj * Wj[1] + pj);
    fs[2] = sa * Wj[2] + hv * (uj * Wj[2]);
    fs[3] = sa * Wj[3] + hv * (uj * Wj[3]);
    fs[4] = sa * Wj[4] + hv * (uj * (Wj[4] + pj));
    P[k][0] = L00 * fs[0] + L01 * fs[1] + L02 * fs[2] + L03 * fs[3] + L04 * fs[4];
    P[k][1] = fs[2] - vv * fs[0];
    P[k][2] = fs[3] - wv * fs[0];
    P[k][3] = L30 * fs[0] + L31 * fs[1] + L32 * fs[2] + L33 * fs[3] + L34 * fs[4];
    P[k][4] = L40 * fs[0] + L41 * fs[1] + L02 * fs[2] + L03 * fs[3] + L04 * fs[4];
  }
  f2 ff[5];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const f2v r = weno_pair<0>(P[0][i], P[1][i], P[2][i], P[3][i], P[4][i]);
    ff[i] = r.x() + r.y();
  }
  // right eigenvector columns (src/utilities.cpp:318-340)
  out[0] = ff[0] + ff[3] + ff[4];
  out[1] = (u - c) * ff[0] + u * ff[3] + (u + c) * ff[4];
  out[2] = v * ff[0] + ff[1] + v * ff[3] + v * ff[4];
  out[3] = ww * ff[0] + ff[2] + ww * ff[3] + ww * ff[4];
  out[4] = (H - u * c) * ff[0] + v * ff[1] + ww * ff[2] + (half * qsq) * ff[3] + (H + u * c) * ff[4];
}

// Two species at once (two independent reconstruction chains)
template <int WV>
__device__ __forceinline__ void tracer_face_flux_f2v_x2(const FaceState<f2>& S, const f2 (&cv)[6],
                                                        const f2 (&cw)[6], f2& rv, f2& rw) {
  f2v a[5], b[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const f2v h(S.hp[k], S.hm[5 - k]);
    a[k] = f2v(cv[k], cv[5 - k]) * h;
    b[k] = f2v(cw[k], cw[5 - k]) * h;
  }
  const f2v2 r = weno_pair_x2<WV>(a[0], a[1], a[2], a[3], a[4], b[0], b[1], b[2], b[3], b[4]);
  rv = r.a.x() + r.a.y();
  rw = r.b.x() + r.b.y();
}

// Float-float tracer part with both sides paired: pair k holds c_k hp_k (lane x) and
// c_{5-k} hm_{5-k} (lane y).
template <int WV>
__device__ __forceinline__ f2 tracer_face_flux_f2v(const FaceState<f2>& S, const f2 (&cv)[6]) {
  f2v a[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) a[k] = f2v(cv[k], cv[5 - k]) * f2v(S.hp[k], S.hm[5 - k]);
  const f2v r = weno_pair<WV>(a[0], a[1], a[2], a[3], a[4]);
  return r.x() + r.y();
}

}  // namespace gbmv
