// FP64 WENO5 characteristic face flux (the reference's face_flux, src/utilities.cpp:270-479),
// arranged to spend as few FP64 instructions as possible -- on GB300 the FP64 pipe retires
// 2 thread-instructions per SM per cycle, so it, not HBM, bounds this form:
//   * nonlinear weights with ONE division per component and side: with a_k = eps + beta_k,
//     sum_k q_k d_k/a_k^2 / sum_k d_k/a_k^2 = sum_k q_k d_k P_k / sum_k d_k P_k, where
//     P_k = prod_{j != k} a_j^2 (a_k >= 1e-6, so P_k >= 1e-24; it overflows only for split
//     fluxes beyond ~1e37, far outside any state the reference handles);
//   * Lax-Friedrichs splitting folded into one FMA per value (0.5 f +- (0.5 alpha) w), and
//     for the tracers one multiply (c_j * 0.5 (u_j +- alpha));
//   * the sparse rows of the left/right eigenvector matrices applied without the zeros.
// Results equal the reference's to a few ulps of each face flux.
#pragma once

#include "common.cuh"

namespace gbmv {

__device__ __forceinline__ double eos64(double gamma, double rho, double mx, double my, double mz,
                                        double et) {
  return (gamma - 1.0) * (et - (mx * mx + my * my + mz * mz) * 0.5 / rho);
}

__device__ __forceinline__ double sqrt0(double x) { return x <= 0.0 ? 0.0 : sqrt(x); }

// Smoothness indicators of the three candidate stencils of f0..f4 (Jiang-Shu, as the
// reference: beta = 13/12 (second difference)^2 + 1/4 (first-difference combination)^2).
template <typename T>
__device__ __forceinline__ void weno_betas(T f0, T f1, T f2, T f3, T f4, T& bA, T& bB, T& bC) {
  const T b13 = T(13.0 / 12.0), q = T(0.25);
  const T dA = f2 - T(2) * f3 + f4, eA = T(3) * f2 - T(4) * f3 + f4;
  const T dB = f1 - T(2) * f2 + f3, eB = f1 - f3;
  const T dC = f0 - T(2) * f1 + f2, eC = f0 - T(4) * f1 + T(3) * f2;
  bA = b13 * (dA * dA) + q * (eA * eA);
  bB = b13 * (dB * dB) + q * (eB * eB);
  bC = b13 * (dC * dC) + q * (eC * eC);
}

// Convex combination of candidates qA..qC with linear weights (dA, dB, dC) and the
// indicators, one division.
template <typename T>
__device__ __forceinline__ T weno_combine(T bA, T bB, T bC, T qA, T qB, T qC, T dA, T dB, T dC) {
  const T eps = T(1e-6);
  T aA = eps + bA, aB = eps + bB, aC = eps + bC;
  aA = aA * aA;
  aB = aB * aB;
  aC = aC * aC;
  const T tA = dA * (aB * aC), tB = dB * (aA * aC), tC = dC * (aA * aB);
  return (tA * qA + tB * qB + tC * qC) / (tA + tB + tC);
}

// Upwind-biased reconstruction at x_{i+1/2} from f0..f4 = points i-2..i+2 (linear weights
// 0.3, 0.6, 0.1 for candidates {f2,f3,f4}, {f1,f2,f3}, {f0,f1,f2}).
__device__ __forceinline__ double weno_plus64(double f0, double f1, double f2, double f3,
                                              double f4) {
  double bA, bB, bC;
  weno_betas(f0, f1, f2, f3, f4, bA, bB, bC);
  const double qA = (1.0 / 3.0) * f2 + (5.0 / 6.0) * f3 - (1.0 / 6.0) * f4;
  const double qB = -(1.0 / 6.0) * f1 + (5.0 / 6.0) * f2 + (1.0 / 3.0) * f3;
  const double qC = (1.0 / 3.0) * f0 - (7.0 / 6.0) * f1 + (11.0 / 6.0) * f2;
  return weno_combine(bA, bB, bC, qA, qB, qC, 0.3, 0.6, 0.1);
}

// Mirror image for the left-moving part, f0..f4 = points i-1..i+3.
__device__ __forceinline__ double weno_minus64(double f0, double f1, double f2, double f3,
                                               double f4) {
  double bA, bB, bC;
  weno_betas(f0, f1, f2, f3, f4, bA, bB, bC);
  const double qA = (11.0 / 6.0) * f2 - (7.0 / 6.0) * f3 + (1.0 / 3.0) * f4;
  const double qB = (1.0 / 3.0) * f1 + (5.0 / 6.0) * f2 - (1.0 / 6.0) * f3;
  const double qC = -(1.0 / 6.0) * f0 + (5.0 / 6.0) * f1 + (1.0 / 3.0) * f2;
  return weno_combine(bA, bB, bC, qA, qB, qC, 0.1, 0.6, 0.3);
}

// Face-local data shared by the fluid and tracer parts.
struct FaceState {
  double hp[6], hm[6];  // 0.5 (u_j + alpha), 0.5 (u_j - alpha): tracer split-flux factors
};

// Fluid part: W[j] = (rho, m_normal, m_t1, m_t2, et) of stencil point j (after the direction
// swap); writes the five fluxes in the same order.
__device__ __forceinline__ void fluid_face_flux64(const double (&W)[6][5], double gamma,
                                                  FaceState& S, double (&out)[5]) {
  double p[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) p[j] = eos64(gamma, W[j][0], W[j][1], W[j][2], W[j][3], W[j][4]);
  // Roe average at the face (src/utilities.cpp:298-304)
  const double sL = sqrt0(W[2][0]), sR = sqrt0(W[3][0]);
  const double sbar = 0.5 * (sL + sR);
  const double u = 0.5 * (W[2][1] / sL + W[3][1] / sR) / sbar;
  const double v = 0.5 * (W[2][2] / sL + W[3][2] / sR) / sbar;
  const double ww = 0.5 * (W[2][3] / sL + W[3][3] / sR) / sbar;
  const double H = 0.5 * ((p[2] + W[2][4]) / sL + (p[3] + W[3][4]) / sR) / sbar;
  const double qsq = u * u + v * v + ww * ww;
  const double gm = gamma - 1.0;
  const double c = gm * (H - 0.5 * qsq);  // the reference's "csnd" (src/utilities.cpp:309)
  const double ci = 1.0 / c;
  // nonzero entries of the left eigenvector rows (src/utilities.cpp:342-364)
  const double hgc = 0.5 * gm * ci, hc = 0.5 * ci;
  const double L00 = hc * (u + 0.5 * gm * qsq), L01 = -hc * (gm * u + 1.0), L02 = -v * hgc,
               L03 = -ww * hgc, L04 = hgc;
  const double gc = gm * ci;
  const double L30 = -gc * (qsq - H), L31 = u * gc, L32 = v * gc, L33 = ww * gc, L34 = -gc;
  const double L40 = -hc * (u - 0.5 * gm * qsq), L41 = -hc * (gm * u - 1.0);

  // point fluxes (halved) and the Lax-Friedrichs speed (src/utilities.cpp:368-380)
  double hf[6][5];
  double alpha = 0.0;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double uj = W[j][1] / W[j][0];
    hf[j][0] = 0.5 * W[j][1];
    hf[j][1] = 0.5 * (uj * W[j][1] + p[j]);
    hf[j][2] = 0.5 * (uj * W[j][2]);
    hf[j][3] = 0.5 * (uj * W[j][3]);
    hf[j][4] = 0.5 * (uj * (W[j][4] + p[j]));
    S.hp[j] = uj;  // temporarily u_j
    const double s = fabs(uj) + sqrt0(gamma * p[j] / W[j][0]);
    alpha = (alpha < s) ? s : alpha;
  }
  const double ha = 0.5 * alpha;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double uj = S.hp[j];
    S.hp[j] = 0.5 * uj + ha;
    S.hm[j] = 0.5 * uj - ha;
  }

  double ff[5];
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    double pr[5][5];  // projected split flux [point][characteristic component]
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const int pt = j + side;
      const double sa = side == 0 ? ha : -ha;
      double fs[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) fs[m] = fma(sa, W[pt][m], hf[pt][m]);
      pr[j][0] = L00 * fs[0] + L01 * fs[1] + L02 * fs[2] + L03 * fs[3] + L04 * fs[4];
      pr[j][1] = fs[2] - v * fs[0];
      pr[j][2] = fs[3] - ww * fs[0];
      pr[j][3] = L30 * fs[0] + L31 * fs[1] + L32 * fs[2] + L33 * fs[3] + L34 * fs[4];
      pr[j][4] = L40 * fs[0] + L41 * fs[1] + L02 * fs[2] + L03 * fs[3] + L04 * fs[4];
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      if (side == 0)
        ff[i] = weno_plus64(pr[0][i], pr[1][i], pr[2][i], pr[3][i], pr[4][i]);
      else
        ff[i] += weno_minus64(pr[0][i], pr[1][i], pr[2][i], pr[3][i], pr[4][i]);
    }
  }
  // right eigenvector columns (src/utilities.cpp:318-340)
  out[0] = ff[0] + ff[3] + ff[4];
  out[1] = (u - c) * ff[0] + u * ff[3] + (u + c) * ff[4];
  out[2] = v * ff[0] + ff[1] + v * ff[3] + v * ff[4];
  out[3] = ww * ff[0] + ff[2] + ww * ff[3] + ww * ff[4];
  out[4] = (H - u * c) * ff[0] + v * ff[1] + ww * ff[2] + (0.5 * qsq) * ff[3] + (H + u * c) * ff[4];
}

// Tracer part for one advected field from its 6 stencil values.
__device__ __forceinline__ double tracer_face_flux64(const FaceState& S, const double (&cv)[6]) {
  double r = weno_plus64(cv[0] * S.hp[0], cv[1] * S.hp[1], cv[2] * S.hp[2], cv[3] * S.hp[3],
                         cv[4] * S.hp[4]);
  r += weno_minus64(cv[1] * S.hm[1], cv[2] * S.hm[2], cv[3] * S.hm[3], cv[4] * S.hm[4],
                    cv[5] * S.hm[5]);
  return r;
}

}  // namespace gbmv
