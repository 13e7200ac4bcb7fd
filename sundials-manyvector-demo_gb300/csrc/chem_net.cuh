// Primordial chemistry network (10 species: H2I, H2II, HI, HII, HM, HeI, HeII, HeIII, de, ge):
// rate interpolation, temperature solve, species sources and the analytic Jacobian, as
// device functions shared by the RHS, Jacobian and fused Newton kernels.
//
// Follows src/raja_primordial_network.cpp (the Dengo "cvklu" network): temperature
// 908-1011, rate interpolation 1044-1248, sources 1305-1375, Jacobian 1518-1867.  The species
// sources are written as reaction fluxes times net stoichiometry, summed in reaction order,
// which is the reference's sum term by term.
#pragma once

#include "common.cuh"
#include "df64.cuh"

namespace gbmv {

constexpr int kNT = 50;      // tables per bin
constexpr int kNRates = 46;  // interpolated per cell (21 rates + 25 cooling terms)
constexpr int kTSize = 1024;

// table rows (order of h5tables.TABLE_NAMES)
enum : int {
  K01, K02, K03, K04, K05, K06, K07, K08, K09, K10, K11, K12, K13, K14, K15, K16, K17, K18, K19,
  K21, K22,
  BREM, CEHEI, CEHEII, CEHI, CIECO, CIHEI, CIHEII, CIHEIS, CIHI, COMPTON, GAEL, GAH2, GAHE, GAHI,
  GAHP, H2LTE, H2MCOOL, H2MHEAT, NCRD1, NCRD2, NCRN, REHEII1, REHEII2, REHEIII, REHII,
  GAMMAH2_1, DGAMMAH2_1, GAMMAH2_2, DGAMMAH2_2
};

struct ChemParams {
  const double* tab;  // device, bin-major: tab[bin * kNT + row]
  // dtab[bin * kNT + row] = tab[(bin + 1) * kNT + row] - tab[bin * kNT + row]: the FP64
  // difference every interpolation in the bin takes, formed once at setup (same rounding)
  const double* dtab;
  // the four H2 adiabatic-index tables for the FP32 temperature iterations, per bin:
  // (float) value and (float)(next - value) of gammaH2_2, dgammaH2_2_dT, gammaH2_1,
  // dgammaH2_1_dT -- the roundings the FP32 iterations apply, done once at setup
  const float* gtab;  // device, gtab[bin * 8 + 2 * table + {0 value, 1 slope}]
  double dbin, idbin, lb, tlo, thi, z, zp1_4;
  float dbinf, idbinf, lbf;  // (float) of dbin, idbin, lb
  int nbins;
};

__device__ __forceinline__ int chem_bin(const ChemParams& P, double logT, double& t1, double& t2) {
  int b = (int)(P.idbin * (logT - P.lb));
  if (b <= 0) b = 0;
  else if (b >= P.nbins) b = P.nbins - 1;
  t1 = P.lb + b * P.dbin;
  t2 = P.lb + (b + 1) * P.dbin;
  return b;
}

// cvklu_calculate_temperature: ten Newton iterations from the previous T, then clamp.
__device__ __forceinline__ void chem_temperature(const ChemParams& P, const double (&y)[10],
                                                 double& Ts, double& dTs_ge) {
  const double kb = 1.3806504e-16, mh = 1.67e-24, gm1 = 1.0 / (5.e0 / 3.e0 - 1);
  const double H2_1 = y[0], H2_2 = y[1], H_1 = y[2], H_2 = y[3], H_m0 = y[4], He_1 = y[5],
               He_2 = y[6], He_3 = y[7], de = y[8], ge = y[9];
  const double density = 2.0 * H2_1 + 2.0 * H2_2 + 1.00794 * H_1 + 1.00794 * H_2 +
                         1.00794 * H_m0 + 4.002602 * He_1 + 4.002602 * He_2 + 4.002602 * He_3;
  const double dmh = density * mh;
  double T = Ts, Tnew = 0.0, dge_dT = 0.0;
#pragma unroll 1
  for (int it = 0; it < 10; ++it) {
    T = Ts;
    double t1, t2;
    const double logT = log(Ts);
    const int b = chem_bin(P, logT, t1, t2);
    const double Tdef = (logT - t1) / (t2 - t1);
    const double* lo = P.tab + (long)b * kNT;
    const double* dl = P.dtab + (long)b * kNT;
    const double g2 = lo[GAMMAH2_2] + Tdef * dl[GAMMAH2_2];
    const double dg2 = lo[DGAMMAH2_2] + Tdef * dl[DGAMMAH2_2];
    const double g1 = lo[GAMMAH2_1] + Tdef * dl[GAMMAH2_1];
    const double dg1 = lo[DGAMMAH2_1] + Tdef * dl[DGAMMAH2_1];
    const double i1 = 1.0 / (g1 - 1.0), i2 = 1.0 / (g2 - 1.0);
    const double nsum = H2_1 * i1 + H2_2 * i2 + H_1 * gm1 + H_2 * gm1 + H_m0 * gm1 + He_1 * gm1 +
                        He_2 * gm1 + He_3 * gm1 + gm1 * de;
    dge_dT = T * kb * (-H2_1 * i1 * i1 * dg1 - H2_2 * i2 * i2 * dg2) / dmh + kb * nsum / dmh;
    const double dge = T * kb * nsum / dmh - ge;
    Tnew = T - dge / dge_dT;
    Ts = Tnew;
  }
  Ts = Tnew;
  if (Ts < P.tlo) Ts = P.tlo;
  else if (Ts > P.thi) Ts = P.thi;
  dTs_ge = 1.0 / dge_dT;
}

// The same Newton solve with up to `nfloat` iterations in FP32 (table lookups on float copies
// of the four adiabatic-index tables, value and slope per bin, rounded once at setup exactly
// as the iterations would round the FP64 entries) and 10 - nfloat in FP64 (the fused Newton
// 8 + 2, which keeps the carried temperature within ~1e-16 of the FP64 form's; the DIRK's F
// evaluations 9 + 1, ~1e-10 near a table bin edge, far inside the integration tolerance,
// where Newton converges only linearly).  The FP32 stage stops early
// once its step is below 1e-5 T: Newton's error after such a step is ~1e-10 T, inside the
// basin where the two FP64 iterations restore full accuracy (quadratic convergence), so the
// result matches chem_temperature's to rounding whenever the reference's ten iterations
// converge.  From the carried temperature of a nearby state (successive stages, Newton
// iterates) one FP32 iteration usually suffices.
__device__ __forceinline__ void chem_temperature_mixed(const ChemParams& P, const double (&y)[10],
                                                       double& Ts, double& dTs_ge, int nfloat) {
  const float kb = 1.3806504e-16f, mh = 1.67e-24f, gm1 = 1.5f;
  const float H2_1 = (float)y[0], H2_2 = (float)y[1], H_1 = (float)y[2], H_2 = (float)y[3],
              H_m0 = (float)y[4], He_1 = (float)y[5], He_2 = (float)y[6], He_3 = (float)y[7],
              de = (float)y[8], ge = (float)y[9];
  const float density = 2.f * H2_1 + 2.f * H2_2 + 1.00794f * H_1 + 1.00794f * H_2 +
                        1.00794f * H_m0 + 4.002602f * He_1 + 4.002602f * He_2 + 4.002602f * He_3;
  const float kdm = kb / (density * mh);
  const float lb = P.lbf, idbin = P.idbinf, dbin = P.dbinf;
  float T = (float)Ts;
#pragma unroll 1
  for (int it = 0; it < nfloat; ++it) {
    const float logT = logf(T);
    int b = (int)(idbin * (logT - lb));
    b = b <= 0 ? 0 : (b >= P.nbins ? P.nbins - 1 : b);
    const float t1 = lb + b * dbin;
    const float Tdef = (logT - t1) / dbin;
    const float4 ga = __ldg(reinterpret_cast<const float4*>(P.gtab + (long)b * 8));
    const float4 gb = __ldg(reinterpret_cast<const float4*>(P.gtab + (long)b * 8 + 4));
    const float g2 = ga.x + Tdef * ga.y;
    const float dg2 = ga.z + Tdef * ga.w;
    const float g1 = gb.x + Tdef * gb.y;
    const float dg1 = gb.z + Tdef * gb.w;
    const float i1 = 1.f / (g1 - 1.f), i2 = 1.f / (g2 - 1.f);
    const float nsum = H2_1 * i1 + H2_2 * i2 +
                       gm1 * (H_1 + H_2 + H_m0 + He_1 + He_2 + He_3 + de);
    const float dge_dT = kdm * (T * (-H2_1 * i1 * i1 * dg1 - H2_2 * i2 * i2 * dg2) + nsum);
    const float dge = kdm * T * nsum - ge;
    const float dT = dge / dge_dT;
    T = T - dT;
    if (fabsf(dT) <= 1e-5f * T) break;
  }
  Ts = (double)T;
  // remaining iterations (and dT/dge) in FP64: exactly chem_temperature's loop body
  const double kbd = 1.3806504e-16, mhd = 1.67e-24, gm1d = 1.0 / (5.e0 / 3.e0 - 1);
  const double dH2_1 = y[0], dH2_2 = y[1], dH_1 = y[2], dH_2 = y[3], dH_m0 = y[4], dHe_1 = y[5],
               dHe_2 = y[6], dHe_3 = y[7], dde = y[8], dge0 = y[9];
  const double ddensity = 2.0 * dH2_1 + 2.0 * dH2_2 + 1.00794 * dH_1 + 1.00794 * dH_2 +
                          1.00794 * dH_m0 + 4.002602 * dHe_1 + 4.002602 * dHe_2 + 4.002602 * dHe_3;
  const double dmh = ddensity * mhd;
  // the FP64 tail multiplies by reciprocals where the FP64 form divides (one rounding apart;
  // each FP64 division costs about as much as ten multiplies on this part)
  const double kdmd = kbd / dmh;
  double Tc = Ts, Tnew = Ts, dge_dTd = 0.0;
#pragma unroll 1
  for (int it = nfloat; it < 10; ++it) {
    Tc = Ts;
    double t1, t2;
    const double logT = log(Ts);
    const int b = chem_bin(P, logT, t1, t2);
    const double Tdef = (logT - t1) * P.idbin;
    const double* lo = P.tab + (long)b * kNT;
    const double* dl = P.dtab + (long)b * kNT;
    const double g2 = lo[GAMMAH2_2] + Tdef * dl[GAMMAH2_2];
    const double dg2 = lo[DGAMMAH2_2] + Tdef * dl[DGAMMAH2_2];
    const double g1 = lo[GAMMAH2_1] + Tdef * dl[GAMMAH2_1];
    const double dg1 = lo[DGAMMAH2_1] + Tdef * dl[DGAMMAH2_1];
    const double i1 = 1.0 / (g1 - 1.0), i2 = 1.0 / (g2 - 1.0);
    const double nsum = dH2_1 * i1 + dH2_2 * i2 + dH_1 * gm1d + dH_2 * gm1d + dH_m0 * gm1d +
                        dHe_1 * gm1d + dHe_2 * gm1d + dHe_3 * gm1d + gm1d * dde;
    dge_dTd = kdmd * (Tc * (-dH2_1 * i1 * i1 * dg1 - dH2_2 * i2 * i2 * dg2) + nsum);
    const double dgev = kdmd * Tc * nsum - dge0;
    Tnew = Tc - dgev / dge_dTd;
    Ts = Tnew;
  }
  Ts = Tnew;
  if (Ts < P.tlo) Ts = P.tlo;
  else if (Ts > P.thi) Ts = P.thi;
  dTs_ge = 1.0 / dge_dTd;
}

// Rates at temperature Ts (and their T-derivatives when WithSlopes).  Reciprocal: the
// interpolation weight and the slope factor multiply by 1 / dbin instead of dividing by the
// bin width t2 - t1 (one division per cell instead of three, within an ulp or two of the
// quotients; the mixed forms' choice -- the FP64 forms divide, as the reference does).
template <bool WithSlopes, bool Reciprocal = false>
__device__ __forceinline__ void chem_rates(const ChemParams& P, double Ts, double (&k)[kNRates],
                                           double (&dk)[kNRates]) {
  double t1, t2;
  const double logT = log(Ts);
  const int b = chem_bin(P, logT, t1, t2);
  const double Tdef = Reciprocal ? (logT - t1) * P.idbin : (logT - t1) / (t2 - t1);
  const double Tfactor = Reciprocal ? P.idbin / Ts : (1.0 / Ts) / (t2 - t1);
  const double* lo = P.tab + (long)b * kNT;
  const double* dl = P.dtab + (long)b * kNT;
#pragma unroll
  for (int r = 0; r < kNRates; ++r) {
    const double a = __ldg(lo + r), d = __ldg(dl + r);
    k[r] = a + Tdef * d;
    if (WithSlopes) dk[r] = d * Tfactor;
  }
}

// The 21 reaction fluxes (rate times reactant product).
__device__ __forceinline__ void chem_fluxes(const double (&k)[kNRates], const double (&y)[10],
                                            double (&r)[21]) {
  const double H2_1 = y[0], H2_2 = y[1], H_1 = y[2], H_2 = y[3], H_m0 = y[4], He_1 = y[5],
               He_2 = y[6], He_3 = y[7], de = y[8];
  r[0] = k[K01] * H_1 * de;
  r[1] = k[K02] * H_2 * de;
  r[2] = k[K03] * He_1 * de;
  r[3] = k[K04] * He_2 * de;
  r[4] = k[K05] * He_2 * de;
  r[5] = k[K06] * He_3 * de;
  r[6] = k[K07] * H_1 * de;
  r[7] = k[K08] * H_1 * H_m0;
  r[8] = k[K09] * H_1 * H_2;
  r[9] = k[K10] * H2_2 * H_1;
  r[10] = k[K11] * H2_1 * H_2;
  r[11] = k[K12] * H2_1 * de;
  r[12] = k[K13] * H2_1 * H_1;
  r[13] = k[K14] * H_m0 * de;
  r[14] = k[K15] * H_1 * H_m0;
  r[15] = k[K16] * H_2 * H_m0;
  r[16] = k[K17] * H_2 * H_m0;
  r[17] = k[K18] * H2_2 * de;
  r[18] = k[K19] * H2_2 * H_m0;
  r[19] = k[K21] * H2_1 * H_1 * H_1;
  r[20] = k[K22] * H_1 * H_1 * H_1;
}

// Net species sources from reaction fluxes (net stoichiometry, reaction order).
__device__ __forceinline__ void chem_species(const double (&r)[21], double (&s)[9]) {
  s[0] = r[7] + r[9] - r[10] - r[11] - r[12] + r[18] + r[19] + r[20];
  s[1] = r[8] - r[9] + r[10] + r[16] - r[17] - r[18];
  s[2] = -r[0] + r[1] - r[6] - r[7] - r[8] - r[9] + r[10] + 2 * r[11] + 2 * r[12] + r[13] + r[14] +
         2 * r[15] + 2 * r[17] + r[18] - 2 * r[19] - 2 * r[20];
  s[3] = r[0] - r[1] - r[8] + r[9] - r[10] - r[15] - r[16];
  s[4] = r[6] - r[7] - r[13] - r[14] - r[15] - r[16] - r[18];
  s[5] = -r[2] + r[3];
  s[6] = r[2] - r[3] - r[4] + r[5];
  s[7] = r[4] - r[5];
  s[8] = r[0] - r[1] + r[2] - r[3] + r[4] - r[5] - r[6] + r[7] + r[13] + r[14] + r[16] - r[17];
}

struct ChemAux {
  double mdens, imdens, cie, h2;
};

// Gas-energy source (cooling/heating), src/raja_primordial_network.cpp:1371-1375.
__device__ __forceinline__ double chem_ge_source(const ChemParams& P, const double (&k)[kNRates],
                                                 const double (&y)[10], double T,
                                                 const ChemAux& A) {
  const double H2_1 = y[0], H_1 = y[2], H_2 = y[3], He_1 = y[5], He_2 = y[6], He_3 = y[7],
               de = y[8];
  const double z = P.z, cie = A.cie, h2oda = A.h2, mdens = A.mdens;
  const double G = H2_1 * k[GAH2] + H_1 * k[GAHI] + H_2 * k[GAHP] + He_1 * k[GAHE] + de * k[GAEL];
  const double D = k[H2LTE] / G + 1.0;
  const double F = k[NCRN] / (H2_1 * k[NCRD2] + H_1 * k[NCRD1]) + 1.0;
  const double H13 = H_1 * H_1 * H_1;
  const double Hf = -H2_1 * H_1 * k[H2MCOOL] + H13 * k[H2MHEAT];
  const double de2 = de * de;
  return -2.01588 * H2_1 * k[CIECO] * cie * mdens - H2_1 * cie * k[H2LTE] * h2oda / D -
         H_1 * k[CEHI] * cie * de - H_1 * k[CIHI] * cie * de - H_2 * cie * de * k[REHII] -
         He_1 * k[CIHEI] * cie * de - He_2 * k[CEHEII] * cie * de - He_2 * k[CEHEI] * cie * de2 -
         He_2 * k[CIHEII] * cie * de - He_2 * k[CIHEIS] * cie * de2 -
         He_2 * cie * de * k[REHEII1] - He_2 * cie * de * k[REHEII2] -
         He_3 * cie * de * k[REHEIII] - k[BREM] * cie * de * (H_2 + He_2 + 4.0 * He_3) -
         cie * k[COMPTON] * de * P.zp1_4 * (T - 2.73 * z - 2.73) + 0.5 / F * Hf;
}

// The four reciprocals of the cooling/heating terms (1/G, 1/D, 1/N, 1/F), shared by the gas-
// energy source and its Jacobian row when both are evaluated together.
struct GeRecip {
  double iG, iD, iN, iF;
};
__device__ __forceinline__ GeRecip ge_recip(const double (&k)[kNRates], const double (&y)[10]) {
  const double H2_1 = y[0], H_1 = y[2], H_2 = y[3], He_1 = y[5], de = y[8];
  GeRecip r;
  const double G = H2_1 * k[GAH2] + H_1 * k[GAHI] + H_2 * k[GAHP] + He_1 * k[GAHE] + de * k[GAEL];
  r.iG = 1.0 / G;
  r.iD = 1.0 / (k[H2LTE] * r.iG + 1.0);
  r.iN = 1.0 / (H2_1 * k[NCRD2] + H_1 * k[NCRD1]);
  r.iF = 1.0 / (k[NCRN] * r.iN + 1.0);
  return r;
}

// chem_ge_source with the shared reciprocals (the fused kernels: one rounding apart from the
// reference's divisions).
__device__ __forceinline__ double chem_ge_source_r(const ChemParams& P, const double (&k)[kNRates],
                                                   const double (&y)[10], double T,
                                                   const ChemAux& A, const GeRecip& R) {
  const double H2_1 = y[0], H_1 = y[2], H_2 = y[3], He_1 = y[5], He_2 = y[6], He_3 = y[7],
               de = y[8];
  const double z = P.z, cie = A.cie, h2oda = A.h2, mdens = A.mdens;
  const double H13 = H_1 * H_1 * H_1;
  const double Hf = -H2_1 * H_1 * k[H2MCOOL] + H13 * k[H2MHEAT];
  const double de2 = de * de;
  return -2.01588 * H2_1 * k[CIECO] * cie * mdens - H2_1 * cie * k[H2LTE] * h2oda * R.iD -
         H_1 * k[CEHI] * cie * de - H_1 * k[CIHI] * cie * de - H_2 * cie * de * k[REHII] -
         He_1 * k[CIHEI] * cie * de - He_2 * k[CEHEII] * cie * de - He_2 * k[CEHEI] * cie * de2 -
         He_2 * k[CIHEII] * cie * de - He_2 * k[CIHEIS] * cie * de2 -
         He_2 * cie * de * k[REHEII1] - He_2 * cie * de * k[REHEII2] -
         He_3 * cie * de * k[REHEIII] - k[BREM] * cie * de * (H_2 + He_2 + 4.0 * He_3) -
         cie * k[COMPTON] * de * P.zp1_4 * (T - 2.73 * z - 2.73) + 0.5 * R.iF * Hf;
}

// Analytic Jacobian in physical units, before the inv_scale*scale and time-unit factors;
// rates k and slopes dk at the cell temperature.  Each of the 64 nonzeros is handed to
// put(row, col, value) once, already multiplied by the factors the reference applies to that
// entry (1/mdensity on the ge row, dT/dge on the ge column); entries never put are zero.
// Raw: those two factors are left out, for a caller that folds them into its own row and
// column scaling (one multiply per cell instead of one per entry).
template <bool Raw = false, class Put>
__device__ __forceinline__ void chem_jacobian(const ChemParams& P, const double (&k)[kNRates],
                                              const double (&dk)[kNRates], const double (&y)[10],
                                              double T, double Tge, const ChemAux& A, Put&& put,
                                              const GeRecip* shared = nullptr) {
  const double H2_1 = y[0], H2_2 = y[1], H_1 = y[2], H_2 = y[3], H_m0 = y[4], He_1 = y[5],
               He_2 = y[6], He_3 = y[7], de = y[8];
  const double z = P.z, h2oda = A.h2, md = A.mdens, imd = A.imdens;
#define SETJ(row, col, expr) put(row, col, (expr))
#define SETG(col, expr) put(9, col, Raw ? (expr) : (expr) * imd)
  const double H1sq = H_1 * H_1;
  SETJ(0, 0, -k[K11] * H_2 - k[K12] * de - k[K13] * H_1 + k[K21] * H1sq);
  SETJ(0, 1, k[K10] * H_1 + k[K19] * H_m0);
  SETJ(0, 2, k[K08] * H_m0 + k[K10] * H2_2 - k[K13] * H2_1 + 2 * k[K21] * H2_1 * H_1 +
                 3 * k[K22] * H1sq);
  SETJ(0, 3, -k[K11] * H2_1);
  SETJ(0, 4, k[K08] * H_1 + k[K19] * H2_2);
  SETJ(0, 8, -k[K12] * H2_1);
  SETJ(1, 0, k[K11] * H_2);
  SETJ(1, 1, -k[K10] * H_1 - k[K18] * de - k[K19] * H_m0);
  SETJ(1, 2, k[K09] * H_2 - k[K10] * H2_2);
  SETJ(1, 3, k[K09] * H_1 + k[K11] * H2_1 + k[K17] * H_m0);
  SETJ(1, 4, k[K17] * H_2 - k[K19] * H2_2);
  SETJ(1, 8, -k[K18] * H2_2);
  SETJ(2, 0, k[K11] * H_2 + 2 * k[K12] * de + 2 * k[K13] * H_1 - 2 * k[K21] * H1sq);
  SETJ(2, 1, -k[K10] * H_1 + 2 * k[K18] * de + k[K19] * H_m0);
  SETJ(2, 2, -k[K01] * de - k[K07] * de - k[K08] * H_m0 - k[K09] * H_2 - k[K10] * H2_2 +
                 2 * k[K13] * H2_1 + k[K15] * H_m0 - 4 * k[K21] * H2_1 * H_1 - 6 * k[K22] * H1sq);
  SETJ(2, 3, k[K02] * de - k[K09] * H_1 + k[K11] * H2_1 + 2 * k[K16] * H_m0);
  SETJ(2, 4, -k[K08] * H_1 + k[K14] * de + k[K15] * H_1 + 2 * k[K16] * H_2 + k[K19] * H2_2);
  SETJ(2, 8, -k[K01] * H_1 + k[K02] * H_2 - k[K07] * H_1 + 2 * k[K12] * H2_1 + k[K14] * H_m0 +
                 2 * k[K18] * H2_2);
  SETJ(3, 0, -k[K11] * H_2);
  SETJ(3, 1, k[K10] * H_1);
  SETJ(3, 2, k[K01] * de - k[K09] * H_2 + k[K10] * H2_2);
  SETJ(3, 3, -k[K02] * de - k[K09] * H_1 - k[K11] * H2_1 - k[K16] * H_m0 - k[K17] * H_m0);
  SETJ(3, 4, -k[K16] * H_2 - k[K17] * H_2);
  SETJ(3, 8, k[K01] * H_1 - k[K02] * H_2);
  SETJ(4, 1, -k[K19] * H_m0);
  SETJ(4, 2, k[K07] * de - k[K08] * H_m0 - k[K15] * H_m0);
  SETJ(4, 3, -k[K16] * H_m0 - k[K17] * H_m0);
  SETJ(4, 4, -k[K08] * H_1 - k[K14] * de - k[K15] * H_1 - k[K16] * H_2 - k[K17] * H_2 -
                 k[K19] * H2_2);
  SETJ(4, 8, k[K07] * H_1 - k[K14] * H_m0);
  SETJ(5, 5, -k[K03] * de);
  SETJ(5, 6, k[K04] * de);
  SETJ(5, 8, -k[K03] * He_1 + k[K04] * He_2);
  SETJ(6, 5, k[K03] * de);
  SETJ(6, 6, -k[K04] * de - k[K05] * de);
  SETJ(6, 7, k[K06] * de);
  SETJ(6, 8, k[K03] * He_1 - k[K04] * He_2 - k[K05] * He_2 + k[K06] * He_3);
  SETJ(7, 6, k[K05] * de);
  SETJ(7, 7, -k[K06] * de);
  SETJ(7, 8, k[K05] * He_2 - k[K06] * He_3);
  SETJ(8, 1, -k[K18] * de);
  SETJ(8, 2, k[K01] * de - k[K07] * de + k[K08] * H_m0 + k[K15] * H_m0);
  SETJ(8, 3, -k[K02] * de + k[K17] * H_m0);
  SETJ(8, 4, k[K08] * H_1 + k[K14] * de + k[K15] * H_1 + k[K17] * H_2);
  SETJ(8, 5, k[K03] * de);
  SETJ(8, 6, -k[K04] * de + k[K05] * de);
  SETJ(8, 7, -k[K06] * de);
  SETJ(8, 8, k[K01] * H_1 - k[K02] * H_2 + k[K03] * He_1 - k[K04] * He_2 + k[K05] * He_2 -
                 k[K06] * He_3 - k[K07] * H_1 + k[K14] * H_m0 - k[K18] * H2_2);
  {  // species rows by ge: sources with rates replaced by slopes, times dT/dge
    double r[21], s[9];
    chem_fluxes(dk, y, r);
    chem_species(r, s);
#pragma unroll
    for (int q = 0; q < 9; ++q) put(q, 9, Raw ? s[q] : s[q] * Tge);
  }
  // four reciprocals serve every ge-row entry (the reference divides ~20 times)
  const GeRecip R = shared ? *shared : ge_recip(k, y);
  const double iG = R.iG, iD = R.iD, iN = R.iN, iF = R.iF;
  const double H13 = H1sq * H_1;
  const double Hf = -H2_1 * H_1 * k[H2MCOOL] + H13 * k[H2MHEAT];
  const double lte2 = k[H2LTE] * k[H2LTE];
  const double iDG2 = (iD * iD) * (iG * iG);
  const double iF2 = iF * iF;
  const double iN2 = iN * iN;
  const double lteh = lte2 * h2oda * iDG2;  // h2lte^2 * h2oda / (D^2 G^2)
  SETG(0, -H2_1 * k[GAH2] * lteh - 0.5 * H_1 * k[H2MCOOL] * iF - 2.01588 * k[CIECO] * md -
              k[H2LTE] * h2oda * iD + 0.5 * k[NCRD2] * k[NCRN] * iF2 * Hf * iN2);
  SETG(2, -H2_1 * k[GAHI] * lteh - k[CEHI] * de - k[CIHI] * de +
              0.5 * k[NCRD1] * k[NCRN] * iF2 * Hf * iN2 +
              0.5 * (-H2_1 * k[H2MCOOL] + 3 * H1sq * k[H2MHEAT]) * iF);
  SETG(3, -H2_1 * k[GAHP] * lteh - k[BREM] * de - de * k[REHII]);
  SETG(5, -H2_1 * k[GAHE] * lteh - k[CIHEI] * de);
  SETG(6, -k[BREM] * de - k[CEHEII] * de - k[CEHEI] * (de * de) - k[CIHEII] * de -
              k[CIHEIS] * (de * de) - de * k[REHEII1] - de * k[REHEII2]);
  SETG(7, -4.0 * k[BREM] * de - de * k[REHEIII]);
  SETG(8, -H2_1 * k[GAEL] * lteh - H_1 * k[CEHI] - H_1 * k[CIHI] - H_2 * k[REHII] -
              He_1 * k[CIHEI] - He_2 * k[CEHEII] - 2 * He_2 * k[CEHEI] * de - He_2 * k[CIHEII] -
              2 * He_2 * k[CIHEIS] * de - He_2 * k[REHEII1] - He_2 * k[REHEII2] -
              He_3 * k[REHEIII] - k[BREM] * (H_2 + He_2 + 4.0 * He_3) -
              k[COMPTON] * P.zp1_4 * (T - 2.73 * z - 2.73));
  const double dGn = -H2_1 * dk[GAH2] - H_1 * dk[GAHI] - H_2 * dk[GAHP] - He_1 * dk[GAHE] -
                     de * dk[GAEL];
  const double gg = -H2_1 * k[H2LTE] * h2oda * (-k[H2LTE] * dGn * (iG * iG) - dk[H2LTE] * iG) *
                        (iD * iD) -
                    H2_1 * h2oda * dk[H2LTE] * iD +
                    0.5 * iF2 * Hf *
                        (-1.0 * k[NCRN] * (-H2_1 * dk[NCRD2] - H_1 * dk[NCRD1]) * iN2 -
                         1.0 * dk[NCRN] * iN) +
                    0.5 * iF * (-H2_1 * H_1 * dk[H2MCOOL] + H13 * dk[H2MHEAT]);
  put(9, 9, Raw ? gg : gg * imd * Tge);
#undef SETG
#undef SETJ
}


}  // namespace gbmv
