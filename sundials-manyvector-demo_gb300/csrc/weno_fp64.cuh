// FP64 WENO5 characteristic face flux, in the evaluation order of the reference's face_flux
// (src/utilities.cpp:270-479) so that results agree with it to rounding (FMA contraction is
// the only difference).  Used by the FP64 parity form of the flux divergence.
#pragma once

#include "common.cuh"

namespace gbmv {

struct FluidStencil {
  double w[6][5];  // rho, m_normal, m_t1, m_t2, et after the direction swap
};

__device__ __forceinline__ double eos64(double gamma, double rho, double mx, double my, double mz,
                                        double et) {
  return (gamma - 1.0) * (et - (mx * mx + my * my + mz * mz) * 0.5 / rho);
}

__device__ __forceinline__ double sqrt0(double x) { return x <= 0.0 ? 0.0 : sqrt(x); }

// WENO5-JS upwind-biased reconstruction at x_{i+1/2} from f0..f4 (points i-2..i+2),
// linear weights (0.3, 0.6, 0.1) for candidates (f2f3f4, f1f2f3, f0f1f2), eps = 1e-6.
__device__ __forceinline__ double weno_plus64(double f0, double f1, double f2, double f3,
                                              double f4) {
  const double b13 = 13.0 / 12.0, eps = 1e-6;
  const double dA = f2 - 2.0 * f3 + f4, eA = 3.0 * f2 - 4.0 * f3 + f4;
  const double dB = f1 - 2.0 * f2 + f3, eB = f1 - f3;
  const double dC = f0 - 2.0 * f1 + f2, eC = f0 - 4.0 * f1 + 3.0 * f2;
  const double bA = b13 * (dA * dA) + 0.25 * (eA * eA);
  const double bB = b13 * (dB * dB) + 0.25 * (eB * eB);
  const double bC = b13 * (dC * dC) + 0.25 * (eC * eC);
  const double wA = 0.3 / ((eps + bA) * (eps + bA));
  const double wB = 0.6 / ((eps + bB) * (eps + bB));
  const double wC = 0.1 / ((eps + bC) * (eps + bC));
  const double qA = (1.0 / 3.0) * f2 + (5.0 / 6.0) * f3 - (1.0 / 6.0) * f4;
  const double qB = -(1.0 / 6.0) * f1 + (5.0 / 6.0) * f2 + (1.0 / 3.0) * f3;
  const double qC = (1.0 / 3.0) * f0 - (7.0 / 6.0) * f1 + (11.0 / 6.0) * f2;
  return (qA * wA + qB * wB + qC * wC) / (wA + wB + wC);
}

// Mirror image: reconstruction of the left-moving part from points i-1..i+3 (f0..f4).
__device__ __forceinline__ double weno_minus64(double f0, double f1, double f2, double f3,
                                               double f4) {
  const double b13 = 13.0 / 12.0, eps = 1e-6;
  const double dA = f2 - 2.0 * f3 + f4, eA = 3.0 * f2 - 4.0 * f3 + f4;
  const double dB = f1 - 2.0 * f2 + f3, eB = f1 - f3;
  const double dC = f0 - 2.0 * f1 + f2, eC = f0 - 4.0 * f1 + 3.0 * f2;
  const double bA = b13 * (dA * dA) + 0.25 * (eA * eA);
  const double bB = b13 * (dB * dB) + 0.25 * (eB * eB);
  const double bC = b13 * (dC * dC) + 0.25 * (eC * eC);
  const double wA = 0.1 / ((eps + bA) * (eps + bA));
  const double wB = 0.6 / ((eps + bB) * (eps + bB));
  const double wC = 0.3 / ((eps + bC) * (eps + bC));
  const double qA = (11.0 / 6.0) * f2 - (7.0 / 6.0) * f3 + (1.0 / 3.0) * f4;
  const double qB = (1.0 / 3.0) * f1 + (5.0 / 6.0) * f2 - (1.0 / 6.0) * f3;
  const double qC = -(1.0 / 6.0) * f0 + (5.0 / 6.0) * f1 + (1.0 / 3.0) * f2;
  return (qA * wA + qB * wB + qC * wC) / (wA + wB + wC);
}

// Face-local characteristic data shared by the fluid and tracer parts.
struct FaceState {
  double u, v, w, H, c, ci, gm, qsq;  // Roe state; c is (gamma-1)(H - q^2/2) as in the reference
  double alpha;                       // Lax-Friedrichs speed: max over the 6 points
  double uj[6];                       // normal velocity at each stencil point
};

// Fluid part: fills out[0..4] (direction-independent ordering: rho, m_n, m_t1, m_t2, et)
__device__ __forceinline__ void fluid_face_flux64(const double (&W)[6][5], double gamma,
                                                  FaceState& S, double (&out)[5]) {
  double p[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) p[j] = eos64(gamma, W[j][0], W[j][1], W[j][2], W[j][3], W[j][4]);
  const double sL = sqrt0(W[2][0]), sR = sqrt0(W[3][0]);
  const double sbar = 0.5 * (sL + sR);
  S.u = 0.5 * (W[2][1] / sL + W[3][1] / sR) / sbar;
  S.v = 0.5 * (W[2][2] / sL + W[3][2] / sR) / sbar;
  S.w = 0.5 * (W[2][3] / sL + W[3][3] / sR) / sbar;
  S.H = 0.5 * ((p[2] + W[2][4]) / sL + (p[3] + W[3][4]) / sR) / sbar;
  S.qsq = S.u * S.u + S.v * S.v + S.w * S.w;
  S.gm = gamma - 1.0;
  S.c = S.gm * (S.H - 0.5 * S.qsq);
  S.ci = 1.0 / S.c;
  const double u = S.u, v = S.v, ww = S.w, H = S.H, c = S.c, ci = S.ci, gm = S.gm, qsq = S.qsq;

  // left eigenvectors (rows), src/utilities.cpp:342-364
  const double L00 = 0.5 * ci * (u + 0.5 * gm * qsq), L01 = -0.5 * ci * (gm * u + 1.0),
               L02 = -0.5 * v * gm * ci, L03 = -0.5 * ww * gm * ci, L04 = 0.5 * gm * ci;
  const double L30 = -gm * ci * (qsq - H), L31 = u * gm * ci, L32 = v * gm * ci,
               L33 = ww * gm * ci, L34 = -gm * ci;
  const double L40 = -0.5 * ci * (u - 0.5 * gm * qsq), L41 = -0.5 * ci * (gm * u - 1.0);

  double flux[6][5];
  double alpha = 0.0;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double uj = W[j][1] / W[j][0];
    S.uj[j] = uj;
    flux[j][0] = W[j][1];
    flux[j][1] = uj * W[j][1] + p[j];
    flux[j][2] = uj * W[j][2];
    flux[j][3] = uj * W[j][3];
    flux[j][4] = uj * (W[j][4] + p[j]);
    const double cj = sqrt0(gamma * p[j] / W[j][0]);
    const double s = fabs(uj) + cj;
    alpha = (alpha < s) ? s : alpha;
  }
  S.alpha = alpha;

  double ff[5];
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    double pr[5][5];  // projected split flux [point][characteristic component]
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      double fs[5];
#pragma unroll
      for (int m = 0; m < 5; ++m)
        fs[m] = side == 0 ? 0.5 * (flux[j][m] + alpha * W[j][m])
                          : 0.5 * (flux[j + 1][m] - alpha * W[j + 1][m]);
      pr[j][0] = L00 * fs[0] + L01 * fs[1] + L02 * fs[2] + L03 * fs[3] + L04 * fs[4];
      pr[j][1] = -v * fs[0] + fs[2];
      pr[j][2] = -ww * fs[0] + fs[3];
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
  // right eigenvectors (columns), src/utilities.cpp:318-340
  out[0] = ff[0] + ff[3] + ff[4];
  out[1] = (u - c) * ff[0] + u * ff[3] + (u + c) * ff[4];
  out[2] = v * ff[0] + ff[1] + v * ff[3] + v * ff[4];
  out[3] = ww * ff[0] + ff[2] + ww * ff[3] + ww * ff[4];
  out[4] = (H - u * c) * ff[0] + v * ff[1] + ww * ff[2] + (0.5 * qsq) * ff[3] + (H + u * c) * ff[4];
}

// Tracer part for one advected field given its 6 stencil values.
__device__ __forceinline__ double tracer_face_flux64(const FaceState& S, const double (&cv)[6]) {
  double fl[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) fl[j] = S.uj[j] * cv[j];
  const double a = S.alpha;
  const double p0 = 0.5 * (fl[0] + a * cv[0]), p1 = 0.5 * (fl[1] + a * cv[1]),
               p2 = 0.5 * (fl[2] + a * cv[2]), p3 = 0.5 * (fl[3] + a * cv[3]),
               p4 = 0.5 * (fl[4] + a * cv[4]);
  const double m0 = 0.5 * (fl[1] - a * cv[1]), m1 = 0.5 * (fl[2] - a * cv[2]),
               m2 = 0.5 * (fl[3] - a * cv[3]), m3 = 0.5 * (fl[4] - a * cv[4]),
               m4 = 0.5 * (fl[5] - a * cv[5]);
  double r = weno_plus64(p0, p1, p2, p3, p4);
  r += weno_minus64(m0, m1, m2, m3, m4);
  return r;
}

}  // namespace gbmv
