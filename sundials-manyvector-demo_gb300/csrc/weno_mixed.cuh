// Mixed-precision WENO5 characteristic face flux.
//
// Precision placement (GB300: FP32 FMAs retire 64x faster than FP64 ones):
//   * per-cell pressure: FP64 (eos, one evaluation per cell, before the FP32 copy) -- the
//     total-minus-kinetic energy difference is where single precision would lose digits;
//   * Roe state, eigenvectors, point fluxes, Lax-Friedrichs splitting, characteristic
//     projections, candidate polynomials, back-projection: FP32;
//   * smoothness indicators and nonlinear weights (and the weighted combination): type WT,
//     either native FP64 (`double`) or float-float (`f2`, ~48-bit significand on the FP32
//     pipes);
//   * the flux divergence and every sum that carries conservation: FP64 (divergence kernel).
#pragma once

#include "common.cuh"
#include "df64.cuh"
#include "weno_fp64.cuh"

namespace gbmv {

__device__ __forceinline__ double wt_from(float x, double*) { return (double)x; }
__device__ __forceinline__ f2 wt_from(float x, f2*) { return f2::from(x); }
__device__ __forceinline__ float wt_to_float(double x) { return (float)x; }
__device__ __forceinline__ float wt_to_float(f2 x) { return x.to_float(); }

template <typename WT>
__device__ __forceinline__ float weno_plus_mx(float f0, float f1, float f2_, float f3, float f4) {
  WT* tag = nullptr;
  const float qA = (1.f / 3.f) * f2_ + (5.f / 6.f) * f3 - (1.f / 6.f) * f4;
  const float qB = -(1.f / 6.f) * f1 + (5.f / 6.f) * f2_ + (1.f / 3.f) * f3;
  const float qC = (1.f / 3.f) * f0 - (7.f / 6.f) * f1 + (11.f / 6.f) * f2_;
  WT bA, bB, bC;
  weno_betas<WT>(wt_from(f0, tag), wt_from(f1, tag), wt_from(f2_, tag), wt_from(f3, tag),
                 wt_from(f4, tag), bA, bB, bC);
  return wt_to_float(weno_combine<WT>(bA, bB, bC, wt_from(qA, tag), wt_from(qB, tag),
                                      wt_from(qC, tag), WT(0.3), WT(0.6), WT(0.1)));
}

template <typename WT>
__device__ __forceinline__ float weno_minus_mx(float f0, float f1, float f2_, float f3, float f4) {
  WT* tag = nullptr;
  const float qA = (11.f / 6.f) * f2_ - (7.f / 6.f) * f3 + (1.f / 3.f) * f4;
  const float qB = (1.f / 3.f) * f1 + (5.f / 6.f) * f2_ - (1.f / 6.f) * f3;
  const float qC = -(1.f / 6.f) * f0 + (5.f / 6.f) * f1 + (1.f / 3.f) * f2_;
  WT bA, bB, bC;
  weno_betas<WT>(wt_from(f0, tag), wt_from(f1, tag), wt_from(f2_, tag), wt_from(f3, tag),
                 wt_from(f4, tag), bA, bB, bC);
  return wt_to_float(weno_combine<WT>(bA, bB, bC, wt_from(qA, tag), wt_from(qB, tag),
                                      wt_from(qC, tag), WT(0.1), WT(0.6), WT(0.3)));
}

struct FaceState32 {
  float hp[6], hm[6];
};

__device__ __forceinline__ float sqrt0f(float x) { return x <= 0.f ? 0.f : sqrtf(x); }

// W[j] = (rho, m_normal, m_t1, m_t2, et) and p[j] of stencil point j (after the swap).
template <typename WT>
__device__ __forceinline__ void fluid_face_flux_mx(const float (&W)[6][5], const float (&p)[6],
                                                   float gamma, FaceState32& S, float (&out)[5]) {
  const float sL = sqrt0f(W[2][0]), sR = sqrt0f(W[3][0]);
  const float isL = 1.f / sL, isR = 1.f / sR;
  const float ihs = 1.f / (sL + sR);  // 0.5 / sbar
  const float u = (W[2][1] * isL + W[3][1] * isR) * ihs;
  const float v = (W[2][2] * isL + W[3][2] * isR) * ihs;
  const float ww = (W[2][3] * isL + W[3][3] * isR) * ihs;
  const float H = ((p[2] + W[2][4]) * isL + (p[3] + W[3][4]) * isR) * ihs;
  const float qsq = u * u + v * v + ww * ww;
  const float gm = gamma - 1.f;
  const float c = gm * (H - 0.5f * qsq);
  const float ci = 1.f / c;
  const float hgc = 0.5f * gm * ci, hc = 0.5f * ci;
  const float L00 = hc * (u + 0.5f * gm * qsq), L01 = -hc * (gm * u + 1.f), L02 = -v * hgc,
              L03 = -ww * hgc, L04 = hgc;
  const float gc = gm * ci;
  const float L30 = -gc * (qsq - H), L31 = u * gc, L32 = v * gc, L33 = ww * gc, L34 = -gc;
  const float L40 = -hc * (u - 0.5f * gm * qsq), L41 = -hc * (gm * u - 1.f);

  float hf[6][5];
  float alpha = 0.f;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const float irho = 1.f / W[j][0];
    const float uj = W[j][1] * irho;
    hf[j][0] = 0.5f * W[j][1];
    hf[j][1] = 0.5f * (uj * W[j][1] + p[j]);
    hf[j][2] = 0.5f * (uj * W[j][2]);
    hf[j][3] = 0.5f * (uj * W[j][3]);
    hf[j][4] = 0.5f * (uj * (W[j][4] + p[j]));
    S.hp[j] = uj;
    const float s = fabsf(uj) + sqrt0f(gamma * p[j] * irho);
    alpha = fmaxf(alpha, s);
  }
  const float ha = 0.5f * alpha;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const float uj = S.hp[j];
    S.hp[j] = 0.5f * uj + ha;
    S.hm[j] = 0.5f * uj - ha;
  }
  float ff[5];
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    float pr[5][5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const int pt = j + side;
      const float sa = side == 0 ? ha : -ha;
      float fs[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) fs[m] = fmaf(sa, W[pt][m], hf[pt][m]);
      pr[j][0] = L00 * fs[0] + L01 * fs[1] + L02 * fs[2] + L03 * fs[3] + L04 * fs[4];
      pr[j][1] = fs[2] - v * fs[0];
      pr[j][2] = fs[3] - ww * fs[0];
      pr[j][3] = L30 * fs[0] + L31 * fs[1] + L32 * fs[2] + L33 * fs[3] + L34 * fs[4];
      pr[j][4] = L40 * fs[0] + L41 * fs[1] + L02 * fs[2] + L03 * fs[3] + L04 * fs[4];
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      if (side == 0)
        ff[i] = weno_plus_mx<WT>(pr[0][i], pr[1][i], pr[2][i], pr[3][i], pr[4][i]);
      else
        ff[i] += weno_minus_mx<WT>(pr[0][i], pr[1][i], pr[2][i], pr[3][i], pr[4][i]);
    }
  }
  out[0] = ff[0] + ff[3] + ff[4];
  out[1] = (u - c) * ff[0] + u * ff[3] + (u + c) * ff[4];
  out[2] = v * ff[0] + ff[1] + v * ff[3] + v * ff[4];
  out[3] = ww * ff[0] + ff[2] + ww * ff[3] + ww * ff[4];
  out[4] = (H - u * c) * ff[0] + v * ff[1] + ww * ff[2] + (0.5f * qsq) * ff[3] + (H + u * c) * ff[4];
}

template <typename WT>
__device__ __forceinline__ float tracer_face_flux_mx(const FaceState32& S, const float (&cv)[6]) {
  float r = weno_plus_mx<WT>(cv[0] * S.hp[0], cv[1] * S.hp[1], cv[2] * S.hp[2], cv[3] * S.hp[3],
                             cv[4] * S.hp[4]);
  r += weno_minus_mx<WT>(cv[1] * S.hm[1], cv[2] * S.hm[2], cv[3] * S.hm[3], cv[4] * S.hm[4],
                         cv[5] * S.hm[5]);
  return r;
}

}  // namespace gbmv
