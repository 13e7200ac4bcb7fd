// Derivatives of the WENO flux divergence (the FP64 form of fEuler, src/utilities.cpp:17-253):
//   VJP  u = (d fEuler / d w)^T v : reverse mode, hand-written.  Per face: the face cotangent
//        from the divergence, cF = (v_{i} - v_{i-1}) / dx along the face normal, then the
//        adjoint of the characteristic face flux (Roe average, eigenvectors, Lax-Friedrichs
//        splitting, WENO5 weights, back-projection) gives the cotangents of the six stencil
//        points, with the direction swap and the ghost signs undone; these are stored per face
//        and stencil slot and a per-cell gather (inverse of the ghost rule, so no atomics and a
//        deterministic result) sums them into u.
// The external forcing is constant in w, so it has no derivative.  Kinks (max over the
// stencil of |u| + c, |u|, the positivity guard of sqrt) take the branch the forward pass took.
#include "common.cuh"
#include "weno.cuh"
#include "weno_face.cuh"
#include "weno_sweep.cuh"

namespace gbmv {

// ------------------------------------------------------------------ VJP

// Reverse sweep of the WENO5 reconstruction weno_side<Plus, double>: fb += (dr/df)^T rb.
template <bool Plus>
__device__ __forceinline__ void weno_side_adj(const double (&f)[5], double rb, double (&fb)[5]) {
  const double dA = f[2] - 2.0 * f[3] + f[4], eA = 3.0 * f[2] - 4.0 * f[3] + f[4];
  const double dB = f[1] - 2.0 * f[2] + f[3], eB = f[1] - f[3];
  const double dC = f[0] - 2.0 * f[1] + f[2], eC = f[0] - 4.0 * f[1] + 3.0 * f[2];
  const double aA = 1e-6 + ((13.0 / 12.0) * (dA * dA) + 0.25 * (eA * eA));
  const double aB = 1e-6 + ((13.0 / 12.0) * (dB * dB) + 0.25 * (eB * eB));
  const double aC = 1e-6 + ((13.0 / 12.0) * (dC * dC) + 0.25 * (eC * eC));
  // candidate polynomials and linear weights (coefficients of f0..f4)
  const double c13 = 1.0 / 3.0, c56 = 5.0 / 6.0, c16 = 1.0 / 6.0, c76 = 7.0 / 6.0,
               c116 = 11.0 / 6.0;
  double QA[5], QB[5], QC[5], wA, wB, wC;
  if (Plus) {
    const double a[5] = {0.0, 0.0, c13, c56, -c16}, b[5] = {0.0, -c16, c56, c13, 0.0},
                 c[5] = {c13, -c76, c116, 0.0, 0.0};
#pragma unroll
    for (int m = 0; m < 5; ++m) { QA[m] = a[m]; QB[m] = b[m]; QC[m] = c[m]; }
    wA = 0.3; wB = 0.6; wC = 0.1;
  } else {
    const double a[5] = {0.0, 0.0, c116, -c76, c13}, b[5] = {0.0, c13, c56, -c16, 0.0},
                 c[5] = {-c16, c56, c13, 0.0, 0.0};
#pragma unroll
    for (int m = 0; m < 5; ++m) { QA[m] = a[m]; QB[m] = b[m]; QC[m] = c[m]; }
    wA = 0.1; wB = 0.6; wC = 0.3;
  }
  double qA = 0.0, qB = 0.0, qC = 0.0;
#pragma unroll
  for (int m = 0; m < 5; ++m) {
    qA += QA[m] * f[m];
    qB += QB[m] * f[m];
    qC += QC[m] * f[m];
  }
  const double tA = wA / (aA * aA), tB = wB / (aB * aB), tC = wC / (aC * aC);
  const double S = tA + tB + tC, iS = 1.0 / S;
  const double r = (tA * qA + tB * qB + tC * qC) * iS;
  // r = sum w_k q_k, w_k = t_k / S;  dr/dq_k = w_k;  dr/dt_k = (q_k - r) / S;
  // t_k = d_k / a_k^2 -> dt_k/da_k = -2 t_k / a_k;  a_k = eps + 13/12 d^2 + 1/4 e^2
  const double gA = rb * (qA - r) * iS * (-2.0 * tA / aA);
  const double gB = rb * (qB - r) * iS * (-2.0 * tB / aB);
  const double gC = rb * (qC - r) * iS * (-2.0 * tC / aC);
  const double wqA = rb * tA * iS, wqB = rb * tB * iS, wqC = rb * tC * iS;
  const double DA[5] = {0.0, 0.0, 1.0, -2.0, 1.0}, EA[5] = {0.0, 0.0, 3.0, -4.0, 1.0};
  const double DB[5] = {0.0, 1.0, -2.0, 1.0, 0.0}, EB[5] = {0.0, 1.0, 0.0, -1.0, 0.0};
  const double DC[5] = {1.0, -2.0, 1.0, 0.0, 0.0}, EC[5] = {1.0, -4.0, 3.0, 0.0, 0.0};
  const double kdA = gA * (13.0 / 6.0) * dA, keA = gA * 0.5 * eA;
  const double kdB = gB * (13.0 / 6.0) * dB, keB = gB * 0.5 * eB;
  const double kdC = gC * (13.0 / 6.0) * dC, keC = gC * 0.5 * eC;
#pragma unroll
  for (int m = 0; m < 5; ++m)
    fb[m] += wqA * QA[m] + wqB * QB[m] + wqC * QC[m] + kdA * DA[m] + keA * EA[m] + kdB * DB[m] +
             keB * EB[m] + kdC * DC[m] + keC * EC[m];
}

// Adjoint of fluid_face_flux<double> + tracer_face_flux<double> for one face.
//   W[6][5]  stencil (face order, signed), ob[5] cotangent of the five fluid fluxes (face
//   order).  Tracers are handled by the caller through hpb/hmb (cotangents of the split
//   factors 0.5 (u_j +- alpha)); this returns Wb[6][5] += the fluid-state cotangents.
struct FluidFwd {
  double p[6], uj[6], sL, sR, sbar, u, v, ww, H, qsq, c, ci;
  double L00, L01, L02, L03, L04, L30, L31, L32, L33, L34, L40, L41;
  double hc, hgc, gc, alpha, ha;
  int amax;
};

__device__ __forceinline__ void fluid_forward(const double (&W)[6][5], double gamma, FluidFwd& F) {
  const double gm = gamma - 1.0;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    F.p[j] = eos_t(gm, W[j][0], W[j][1], W[j][2], W[j][3], W[j][4]);
    F.uj[j] = W[j][1] / W[j][0];
  }
  F.sL = sqrt0(W[2][0]);
  F.sR = sqrt0(W[3][0]);
  F.sbar = 0.5 * (F.sL + F.sR);
  F.u = 0.5 * (W[2][1] / F.sL + W[3][1] / F.sR) / F.sbar;
  F.v = 0.5 * (W[2][2] / F.sL + W[3][2] / F.sR) / F.sbar;
  F.ww = 0.5 * (W[2][3] / F.sL + W[3][3] / F.sR) / F.sbar;
  F.H = 0.5 * ((F.p[2] + W[2][4]) / F.sL + (F.p[3] + W[3][4]) / F.sR) / F.sbar;
  F.qsq = F.u * F.u + F.v * F.v + F.ww * F.ww;
  F.c = gm * (F.H - 0.5 * F.qsq);
  F.ci = 1.0 / F.c;
  F.hgc = 0.5 * gm * F.ci;
  F.hc = 0.5 * F.ci;
  F.gc = gm * F.ci;
  const double u = F.u, v = F.v, ww = F.ww, qsq = F.qsq, H = F.H;
  F.L00 = F.hc * (u + 0.5 * gm * qsq);
  F.L01 = -F.hc * (gm * u + 1.0);
  F.L02 = -v * F.hgc;
  F.L03 = -ww * F.hgc;
  F.L04 = F.hgc;
  F.L30 = -F.gc * (qsq - H);
  F.L31 = u * F.gc;
  F.L32 = v * F.gc;
  F.L33 = ww * F.gc;
  F.L34 = -F.gc;
  F.L40 = -F.hc * (u - 0.5 * gm * qsq);
  F.L41 = -F.hc * (gm * u - 1.0);
  double alpha = 0.0;
  int am = 0;
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double s = fabs(F.uj[j]) + sqrt0(gamma * F.p[j] / W[j][0]);
    if (alpha < s) { alpha = s; am = j; }
  }
  F.alpha = alpha;
  F.amax = am;
  F.ha = 0.5 * alpha;
}

__device__ __forceinline__ void split_point(const FluidFwd& F, const double (&W)[6][5], int pt,
                                            double sa, double (&fs)[5]) {
  const double uj = F.uj[pt], p = F.p[pt];
  const double hf[5] = {0.5 * W[pt][1], 0.5 * (uj * W[pt][1] + p), 0.5 * (uj * W[pt][2]),
                        0.5 * (uj * W[pt][3]), 0.5 * (uj * (W[pt][4] + p))};
#pragma unroll
  for (int m = 0; m < 5; ++m) fs[m] = fma(sa, W[pt][m], hf[m]);
}

__device__ __forceinline__ void project(const FluidFwd& F, const double (&fs)[5], double (&pr)[5]) {
  pr[0] = F.L00 * fs[0] + F.L01 * fs[1] + F.L02 * fs[2] + F.L03 * fs[3] + F.L04 * fs[4];
  pr[1] = fs[2] - F.v * fs[0];
  pr[2] = fs[3] - F.ww * fs[0];
  pr[3] = F.L30 * fs[0] + F.L31 * fs[1] + F.L32 * fs[2] + F.L33 * fs[3] + F.L34 * fs[4];
  pr[4] = F.L40 * fs[0] + F.L41 * fs[1] + F.L02 * fs[2] + F.L03 * fs[3] + F.L04 * fs[4];
}

__device__ void fluid_face_adjoint(const double (&W)[6][5], double gamma, const FluidFwd& F,
                                   const double (&ob)[5], const double (&hpb)[6],
                                   const double (&hmb)[6], double (&Wb)[6][5]) {
  const double gm = gamma - 1.0;
  const double u = F.u, v = F.v, ww = F.ww, H = F.H, qsq = F.qsq, c = F.c;
  // forward characteristic values and reconstructions
  double pr[2][5][5], ff[5];
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const double sa = side == 0 ? F.ha : -F.ha;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      double fs[5];
      split_point(F, W, j + side, sa, fs);
      project(F, fs, pr[side][j]);
    }
  }
#pragma unroll
  for (int i = 0; i < 5; ++i)
    ff[i] = weno_side<true>(pr[0][0][i], pr[0][1][i], pr[0][2][i], pr[0][3][i], pr[0][4][i]) +
            weno_side<false>(pr[1][0][i], pr[1][1][i], pr[1][2][i], pr[1][3][i], pr[1][4][i]);
  // back-projection: out = R ff
  double ub = 0.0, vb = 0.0, wwb = 0.0, Hb = 0.0, qb = 0.0, cb = 0.0;
  const double s034 = ff[0] + ff[3] + ff[4], d04 = ff[4] - ff[0];
  ub += ob[1] * s034 + ob[4] * c * d04;
  cb += ob[1] * d04 + ob[4] * u * d04;
  vb += ob[2] * s034 + ob[4] * ff[1];
  wwb += ob[3] * s034 + ob[4] * ff[2];
  Hb += ob[4] * (ff[0] + ff[4]);
  qb += ob[4] * 0.5 * ff[3];
  double ffb[5];
  ffb[0] = ob[0] + ob[1] * (u - c) + ob[2] * v + ob[3] * ww + ob[4] * (H - u * c);
  ffb[1] = ob[2] + ob[4] * v;
  ffb[2] = ob[3] + ob[4] * ww;
  ffb[3] = ob[0] + ob[1] * u + ob[2] * v + ob[3] * ww + ob[4] * (0.5 * qsq);
  ffb[4] = ob[0] + ob[1] * (u + c) + ob[2] * v + ob[3] * ww + ob[4] * (H + u * c);
  // WENO reconstructions, projections, splitting
  double Lb[13] = {0};  // L00 L01 L02 L03 L04 L30 L31 L32 L33 L34 L40 L41, [12] unused
  double hab = 0.0;
  double hfb[6][5] = {{0}};
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    double prb[5][5] = {{0}};
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const double col[5] = {pr[side][0][i], pr[side][1][i], pr[side][2][i], pr[side][3][i],
                             pr[side][4][i]};
      double cb5[5] = {0, 0, 0, 0, 0};
      if (side == 0) weno_side_adj<true>(col, ffb[i], cb5);
      else weno_side_adj<false>(col, ffb[i], cb5);
#pragma unroll
      for (int j = 0; j < 5; ++j) prb[j][i] = cb5[j];
    }
    const double sa = side == 0 ? F.ha : -F.ha;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
      const int pt = j + side;
      double fs[5];
      split_point(F, W, pt, sa, fs);
      const double* b = prb[j];
      Lb[0] += b[0] * fs[0];
      Lb[1] += b[0] * fs[1];
      Lb[2] += (b[0] + b[4]) * fs[2];
      Lb[3] += (b[0] + b[4]) * fs[3];
      Lb[4] += (b[0] + b[4]) * fs[4];
      Lb[5] += b[3] * fs[0];
      Lb[6] += b[3] * fs[1];
      Lb[7] += b[3] * fs[2];
      Lb[8] += b[3] * fs[3];
      Lb[9] += b[3] * fs[4];
      Lb[10] += b[4] * fs[0];
      Lb[11] += b[4] * fs[1];
      vb -= b[1] * fs[0];
      wwb -= b[2] * fs[0];
      double fsb[5];
      fsb[0] = F.L00 * b[0] - v * b[1] - ww * b[2] + F.L30 * b[3] + F.L40 * b[4];
      fsb[1] = F.L01 * b[0] + F.L31 * b[3] + F.L41 * b[4];
      fsb[2] = F.L02 * b[0] + b[1] + F.L32 * b[3] + F.L02 * b[4];
      fsb[3] = F.L03 * b[0] + b[2] + F.L33 * b[3] + F.L03 * b[4];
      fsb[4] = F.L04 * b[0] + F.L34 * b[3] + F.L04 * b[4];
      double sab = 0.0;
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        Wb[pt][m] += sa * fsb[m];
        hfb[pt][m] += fsb[m];
        sab += fsb[m] * W[pt][m];
      }
      hab += side == 0 ? sab : -sab;
    }
  }
  // tracer split factors hp = 0.5 u_j + ha, hm = 0.5 u_j - ha
  double ujb[6], pb[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    ujb[j] = 0.5 * (hpb[j] + hmb[j]);
    hab += hpb[j] - hmb[j];
    pb[j] = 0.0;
  }
  // ha = alpha / 2, alpha = max_j (|u_j| + sqrt0(gamma p_j / rho_j))
  {
    const int j = F.amax;
    const double sb = 0.5 * hab;
    ujb[j] += (F.uj[j] < 0.0 ? -sb : sb);
    const double x = gamma * F.p[j] / W[j][0];
    if (x > 0.0) {
      const double xb = sb * 0.5 / sqrt(x);
      pb[j] += xb * gamma / W[j][0];
      Wb[j][0] -= xb * x / W[j][0];
    }
  }
  // halved point fluxes
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double uj = F.uj[j], p = F.p[j];
    const double* hb = hfb[j];
    Wb[j][1] += 0.5 * hb[0] + 0.5 * uj * hb[1];
    ujb[j] += 0.5 * (hb[1] * W[j][1] + hb[2] * W[j][2] + hb[3] * W[j][3] + hb[4] * (W[j][4] + p));
    pb[j] += 0.5 * (hb[1] + uj * hb[4]);
    Wb[j][2] += 0.5 * uj * hb[2];
    Wb[j][3] += 0.5 * uj * hb[3];
    Wb[j][4] += 0.5 * uj * hb[4];
    // u_j = m_j / rho_j
    Wb[j][1] += ujb[j] / W[j][0];
    Wb[j][0] -= ujb[j] * uj / W[j][0];
  }
  // left eigenvector entries -> (hc, hgc, gc, u, v, ww, qsq, H)
  double hcb = 0.0, hgcb = 0.0, gcb = 0.0;
  hcb += Lb[0] * (u + 0.5 * gm * qsq);
  ub += Lb[0] * F.hc;
  qb += Lb[0] * F.hc * 0.5 * gm;
  hcb -= Lb[1] * (gm * u + 1.0);
  ub -= Lb[1] * F.hc * gm;
  vb -= Lb[2] * F.hgc;
  hgcb -= Lb[2] * v;
  wwb -= Lb[3] * F.hgc;
  hgcb -= Lb[3] * ww;
  hgcb += Lb[4];
  gcb -= Lb[5] * (qsq - H);
  qb -= Lb[5] * F.gc;
  Hb += Lb[5] * F.gc;
  ub += Lb[6] * F.gc;
  gcb += Lb[6] * u;
  vb += Lb[7] * F.gc;
  gcb += Lb[7] * v;
  wwb += Lb[8] * F.gc;
  gcb += Lb[8] * ww;
  gcb -= Lb[9];
  hcb -= Lb[10] * (u - 0.5 * gm * qsq);
  ub -= Lb[10] * F.hc;
  qb += Lb[10] * F.hc * 0.5 * gm;
  hcb -= Lb[11] * (gm * u - 1.0);
  ub -= Lb[11] * F.hc * gm;
  const double cib = 0.5 * hcb + 0.5 * gm * hgcb + gm * gcb;
  cb -= cib * F.ci * F.ci;
  // c = gm (H - qsq / 2)
  Hb += gm * cb;
  qb -= 0.5 * gm * cb;
  // qsq = u^2 + v^2 + ww^2
  ub += 2.0 * u * qb;
  vb += 2.0 * v * qb;
  wwb += 2.0 * ww * qb;
  // Roe averages: X = a/sL + b/sR, value = X / (2 sbar)
  double sLb = 0.0, sRb = 0.0, sbb = 0.0;
  const double ib = 0.5 / F.sbar;
  auto roe = [&](double val, double vb_, double a, double b, double& ab, double& bb) {
    const double Xb = vb_ * ib;
    sbb -= vb_ * val / F.sbar;
    ab += Xb / F.sL;
    sLb -= Xb * a / (F.sL * F.sL);
    bb += Xb / F.sR;
    sRb -= Xb * b / (F.sR * F.sR);
  };
  roe(u, ub, W[2][1], W[3][1], Wb[2][1], Wb[3][1]);
  roe(v, vb, W[2][2], W[3][2], Wb[2][2], Wb[3][2]);
  roe(ww, wwb, W[2][3], W[3][3], Wb[2][3], Wb[3][3]);
  {
    double a2 = 0.0, a3 = 0.0;
    roe(H, Hb, F.p[2] + W[2][4], F.p[3] + W[3][4], a2, a3);
    pb[2] += a2;
    Wb[2][4] += a2;
    pb[3] += a3;
    Wb[3][4] += a3;
  }
  sLb += 0.5 * sbb;
  sRb += 0.5 * sbb;
  if (W[2][0] > 0.0) Wb[2][0] += sLb * 0.5 / F.sL;
  if (W[3][0] > 0.0) Wb[3][0] += sRb * 0.5 / F.sR;
  // p_j = gm (E - (mx^2 + my^2 + mz^2) / (2 rho))
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const double rho = W[j][0];
    const double K = (W[j][1] * W[j][1] + W[j][2] * W[j][2] + W[j][3] * W[j][3]) * 0.5 / rho;
    const double Kb = -gm * pb[j];
    Wb[j][4] += gm * pb[j];
    Wb[j][1] += Kb * W[j][1] / rho;
    Wb[j][2] += Kb * W[j][2] / rho;
    Wb[j][3] += Kb * W[j][3] / rho;
    Wb[j][0] -= Kb * K / rho;
  }
}

// Face cotangents -> per-face stencil cotangents A[(l * NVAR + v) * nfaces + f] (original
// field order, ghost signs applied, so each entry belongs to the source cell of slot l).
template <int NCHEM, int DIR>
__global__ void __launch_bounds__(128) face_flux_vjp_kernel(Grid g, Fields w, Fields vb,
                                                            double* __restrict__ A, long nfaces) {
  constexpr int NV = 5 + NCHEM;
  const long nd = g.n[DIR];
  const long stride[3] = {1, g.n[0], g.n[0] * g.n[1]};
  for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < nfaces;
       f += (long)gridDim.x * blockDim.x) {
    long cell[6], ijk[3];
    bool nall[6], nnorm[6];
    stencil<DIR>(g, f, cell, nall, nnorm, ijk);
    // face cotangent: + v_i / d for the cell above (i < n), - v_{i-1} / d for the one below
    const long id = ijk[DIR];
    const long cup = ijk[0] + g.n[0] * (ijk[1] + g.n[1] * ijk[2]);  // valid when id < nd
    const long cdn = cup - stride[DIR];
    double cF[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double a = 0.0;
      if (id < nd) a += (v < 5) ? vb.f[v][cup] : vb.f[5][(v - 5) + (long)NCHEM * cup];
      if (id >= 1) a -= (v < 5) ? vb.f[v][cdn] : vb.f[5][(v - 5) + (long)NCHEM * cdn];
      cF[v] = a * g.inv_d[DIR];
    }
    double W[6][5];
#pragma unroll
    for (int l = 0; l < 6; ++l) load_point<DIR>(w, cell[l], nall[l], nnorm[l], W[l]);
    FluidFwd F;
    fluid_forward(W, g.gamma, F);
    // tracers first: their cotangents of the split factors feed the fluid adjoint
    double hpb[6] = {0}, hmb[6] = {0};
#pragma unroll 1
    for (int c = 0; c < NCHEM; ++c) {
      const double rb = cF[5 + c];
      double cv[6], gp[5], gmv[5];
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        const double x = __ldg(w.f[5] + c + (long)NCHEM * cell[l]);
        cv[l] = nall[l] ? -x : x;
      }
      double hp[6], hm[6];
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        hp[l] = 0.5 * F.uj[l] + F.ha;
        hm[l] = 0.5 * F.uj[l] - F.ha;
      }
#pragma unroll
      for (int l = 0; l < 5; ++l) {
        gp[l] = cv[l] * hp[l];
        gmv[l] = cv[l + 1] * hm[l + 1];
      }
      double gpb[5] = {0, 0, 0, 0, 0}, gmb[5] = {0, 0, 0, 0, 0};
      weno_side_adj<true>(gp, rb, gpb);
      weno_side_adj<false>(gmv, rb, gmb);
      double cvb[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int l = 0; l < 5; ++l) {
        cvb[l] += gpb[l] * hp[l];
        hpb[l] += gpb[l] * cv[l];
        cvb[l + 1] += gmb[l] * hm[l + 1];
        hmb[l + 1] += gmb[l] * cv[l + 1];
      }
#pragma unroll
      for (int l = 0; l < 6; ++l)
        A[((long)l * NV + 5 + c) * nfaces + f] = nall[l] ? -cvb[l] : cvb[l];
    }
    // fluid: cotangent of the five fluxes in face order
    double ob[5] = {cF[0], cF[1 + DIR], DIR == 1 ? cF[1] : cF[2], DIR == 2 ? cF[1] : cF[3], cF[4]};
    double Wb[6][5] = {{0}};
    fluid_face_adjoint(W, g.gamma, F, ob, hpb, hmb, Wb);
#pragma unroll
    for (int l = 0; l < 6; ++l) {
      double q[5];
      q[0] = Wb[l][0];
      q[4] = Wb[l][4];
      q[1 + DIR] = Wb[l][1];
      if (DIR == 0) { q[2] = Wb[l][2]; q[3] = Wb[l][3]; }
      if (DIR == 1) { q[1] = Wb[l][2]; q[3] = Wb[l][3]; }
      if (DIR == 2) { q[2] = Wb[l][2]; q[1] = Wb[l][3]; }
      if (nall[l]) {
#pragma unroll
        for (int v = 0; v < 5; ++v) q[v] = -q[v];
      }
      if (nnorm[l]) q[1 + DIR] = -q[1 + DIR];
#pragma unroll
      for (int v = 0; v < 5; ++v) A[((long)l * NV + v) * nfaces + f] = q[v];
    }
  }
}

// u (+)= sum over the (face, slot) pairs whose source cell is c of A[(slot, v), face].
// Positions p along DIR whose ghost source is i: p = i, plus the ghost images (periodic
// wrap, lower mirror -1-i, upper shifted copy i+3) that lie in the stencil range [-3, n+2].
template <int NCHEM, int DIR>
__global__ void __launch_bounds__(256) vjp_gather_kernel(Grid g, const double* __restrict__ A,
                                                         Fields u, long nfaces, int first) {
  constexpr int NV = 5 + NCHEM;
  const long nx = g.n[0], ny = g.n[1], nd = g.n[DIR];
  const int blo = g.bc[2 * DIR], bhi = g.bc[2 * DIR + 1];
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < g.ncell;
       c += (long)gridDim.x * blockDim.x) {
    long i0, j0, k0;
    split3(c, nx, ny, i0, j0, k0);
    const long pos[3] = {i0, j0, k0};
    const long id = pos[DIR];
    long cand[4];
    int nc = 0;
    cand[nc++] = id;
    if (blo == GBMV_BC_PERIODIC) {
      if (id - nd >= -3) cand[nc++] = id - nd;
      if (id + nd <= nd + 2) cand[nc++] = id + nd;
    } else {
      if (-1 - id >= -3) cand[nc++] = -1 - id;
      if (id + 3 >= nd && id + 3 <= nd + 2) cand[nc++] = id + 3;
    }
    (void)bhi;
    double acc[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[v] = 0.0;
    for (int q = 0; q < nc; ++q) {
      const long p = cand[q];
#pragma unroll
      for (int l = 0; l < 6; ++l) {
        const long fd = p + 3 - l;  // face index along DIR whose slot l sits at p
        if (fd < 0 || fd > nd) continue;
        long fp[3] = {pos[0], pos[1], pos[2]};
        fp[DIR] = fd;
        const long ex = nx + (DIR == 0), ey = ny + (DIR == 1);
        const long f = fp[0] + ex * (fp[1] + ey * fp[2]);
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[v] += A[((long)l * NV + v) * nfaces + f];
      }
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double* dst = (v < 5) ? (u.f[v] + c) : (u.f[5] + (v - 5) + (long)NCHEM * c);
      *dst = first ? acc[v] : *dst + acc[v];
    }
  }
}

// ------------------------------------------------------------------ launcher

template <int NCHEM>
static int vjp_t(const Grid& g, const Fields& w, const Fields& v, const Fields& out, double* A,
                 cudaStream_t s) {
  long nf[3];
  face_counts(g, nf);
  ProfScope ps("vjp", s);
  face_flux_vjp_kernel<NCHEM, 0><<<sweep_blocks(nf[0], 128), 128, 0, s>>>(g, w, v, A, nf[0]);
  GBMV_LAUNCH_CHECK("face_flux_vjp_kernel<x>");
  vjp_gather_kernel<NCHEM, 0><<<sweep_blocks(g.ncell, 256), 256, 0, s>>>(g, A, out, nf[0], 1);
  GBMV_LAUNCH_CHECK("vjp_gather_kernel<x>");
  face_flux_vjp_kernel<NCHEM, 1><<<sweep_blocks(nf[1], 128), 128, 0, s>>>(g, w, v, A, nf[1]);
  GBMV_LAUNCH_CHECK("face_flux_vjp_kernel<y>");
  vjp_gather_kernel<NCHEM, 1><<<sweep_blocks(g.ncell, 256), 256, 0, s>>>(g, A, out, nf[1], 0);
  GBMV_LAUNCH_CHECK("vjp_gather_kernel<y>");
  face_flux_vjp_kernel<NCHEM, 2><<<sweep_blocks(nf[2], 128), 128, 0, s>>>(g, w, v, A, nf[2]);
  GBMV_LAUNCH_CHECK("face_flux_vjp_kernel<z>");
  vjp_gather_kernel<NCHEM, 2><<<sweep_blocks(g.ncell, 256), 256, 0, s>>>(g, A, out, nf[2], 0);
  GBMV_LAUNCH_CHECK("vjp_gather_kernel<z>");
  return GBMV_OK;
}

size_t feuler_vjp_scratch_doubles(const Grid& g) {
  const long nx = g.n[0], ny = g.n[1], nz = g.n[2];
  long m = (nx + 1) * ny * nz;
  if (nx * (ny + 1) * nz > m) m = nx * (ny + 1) * nz;
  if (nx * ny * (nz + 1) > m) m = nx * ny * (nz + 1);
  return (size_t)6 * (5 + g.nchem) * (size_t)m;
}

int feuler_vjp(const Grid& g, const Fields& w, const Fields& v, const Fields& out, double* A,
               cudaStream_t s) {
  switch (g.nchem) {
    case 0: return vjp_t<0>(g, w, v, out, A, s);
    case 2: return vjp_t<2>(g, w, v, out, A, s);
    case 4: return vjp_t<4>(g, w, v, out, A, s);
    case 6: return vjp_t<6>(g, w, v, out, A, s);
    case 10: return vjp_t<10>(g, w, v, out, A, s);
    default: return GBMV_EUNSUPPORTED;
  }
}

}  // namespace gbmv
