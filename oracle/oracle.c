/* CPU oracle: plain-C restatement of the reference's RHS hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Every routine states the reference lines it
 * restates; arithmetic is written in the reference's evaluation order and the file is built
 * with -ffp-contract=off, so that it agrees with the reference's own CPU build to rounding
 * (checked against tests/golden fixtures made from that build).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define MAXVAR 32
#define STS 6

/* ------------------------------------------------------------------ hydro */

/* Equation of state p = (gamma-1)(et - |m|^2/(2 rho))  (src/euler3D.hpp:1383-1390). */
static double eos(double gamma, double rho, double mx, double my, double mz, double et) {
  return (gamma - 1.0) * (et - (mx * mx + my * my + mz * mz) * 0.5 / rho);
}

/* legal_state bit mask: 1 density, 2 energy, 4 pressure (src/euler3D.hpp:1405-1414). */
static int legal_state(double gamma, double rho, double mx, double my, double mz, double et) {
  int f = 0;
  if (!(rho > 0.0)) f += 1;
  if (!(et > 0.0)) f += 2;
  if (!(eos(gamma, rho, mx, my, mz, et) > 0.0)) f += 4;
  return f;
}

static double rsqrt_or_zero(double x) { return x <= 0.0 ? 0.0 : sqrt(x); }

/* Value of field v at cell position (p[0],p[1],p[2]), at most one coordinate outside the
 * grid.  Ghost rule of ExchangeStart/pack1D_*_bdry (src/euler3D.hpp:577-1166, 1250-1378):
 *   periodic: wrap; lower non-periodic face: mirror cell -1-p; upper non-periodic face:
 *   the shifted copy p-3 (cells n-3..n-1 for ghosts n..n+2);
 *   Neumann: copy; reflecting: negate the momentum normal to the face; Dirichlet: negate all. */
static double field_at(const orc_grid* g, const double* const* w, int v, const long p_in[3]) {
  const long n[3] = {g->nx, g->ny, g->nz};
  long p[3] = {p_in[0], p_in[1], p_in[2]};
  double sign = 1.0;
  for (int a = 0; a < 3; ++a) {
    int bc = -1;
    if (p[a] < 0) {
      bc = g->bc[2 * a];
      p[a] = (bc == ORC_BC_PERIODIC) ? n[a] + p[a] : -1 - p[a];
    } else if (p[a] >= n[a]) {
      bc = g->bc[2 * a + 1];
      p[a] = (bc == ORC_BC_PERIODIC) ? p[a] - n[a] : p[a] - 3;
    }
    if (bc == ORC_BC_DIRICHLET || (bc == ORC_BC_REFLECTING && v == 1 + a)) sign = -sign;
  }
  const long idx = p[0] + g->nx * (p[1] + g->ny * p[2]);
  const double val = (v < 5) ? w[v][idx] : w[5][(v - 5) + (long)g->nchem * idx];
  return sign * val;
}

/* face_flux (src/utilities.cpp:270-479): WENO5-JS characteristic flux at the face between
 * stencil points 2 and 3 of w1d[6][nvar] (Shu 2003), Lax-Friedrichs splitting with the
 * maximum wave speed over the six points, Roe-averaged eigenvectors for the five fluid
 * fields, tracers reconstructed componentwise.  w1d is modified (direction swap). */
void orc_face_flux(const orc_grid* g, double* w1d, int idir, double* f_face) {
  const int nv = 5 + g->nchem;
  const double gamma = g->gamma;
  double p[STS], flux[STS][MAXVAR], fs[STS - 1][MAXVAR], fproj[STS - 1][MAXVAR], ff[MAXVAR];
  double RV[5][5], LV[5][5];
#define W(j, i) w1d[(j) * nv + (i)]
  if (idir > 0)
    for (int j = 0; j < STS; ++j) {
      double t = W(j, 1);
      W(j, 1) = W(j, 1 + idir);
      W(j, 1 + idir) = t;
    }
  for (int j = 0; j < STS; ++j) p[j] = eos(gamma, W(j, 0), W(j, 1), W(j, 2), W(j, 3), W(j, 4));

  /* Roe average at the face */
  const double sL = rsqrt_or_zero(W(2, 0)), sR = rsqrt_or_zero(W(3, 0));
  const double sbar = 0.5 * (sL + sR);
  const double u = 0.5 * (W(2, 1) / sL + W(3, 1) / sR) / sbar;
  const double v = 0.5 * (W(2, 2) / sL + W(3, 2) / sR) / sbar;
  const double ww = 0.5 * (W(2, 3) / sL + W(3, 3) / sR) / sbar;
  const double H = 0.5 * ((p[2] + W(2, 4)) / sL + (p[3] + W(3, 4)) / sR) / sbar;
  const double qsq = u * u + v * v + ww * ww;
  const double gm = gamma - 1.0;
  const double c = gm * (H - 0.5 * qsq); /* the reference uses this (c^2) as "csnd" */
  const double ci = 1.0 / c;
  memset(RV, 0, sizeof RV);
  memset(LV, 0, sizeof LV);
  RV[0][0] = 1.0; RV[0][3] = 1.0; RV[0][4] = 1.0;
  RV[1][0] = u - c; RV[1][3] = u; RV[1][4] = u + c;
  RV[2][0] = v; RV[2][1] = 1.0; RV[2][3] = v; RV[2][4] = v;
  RV[3][0] = ww; RV[3][2] = 1.0; RV[3][3] = ww; RV[3][4] = ww;
  RV[4][0] = H - u * c; RV[4][1] = v; RV[4][2] = ww; RV[4][3] = 0.5 * qsq; RV[4][4] = H + u * c;
  LV[0][0] = 0.5 * ci * (u + 0.5 * gm * qsq);
  LV[0][1] = -0.5 * ci * (gm * u + 1.0);
  LV[0][2] = -0.5 * v * gm * ci;
  LV[0][3] = -0.5 * ww * gm * ci;
  LV[0][4] = 0.5 * gm * ci;
  LV[1][0] = -v; LV[1][2] = 1.0;
  LV[2][0] = -ww; LV[2][3] = 1.0;
  LV[3][0] = -gm * ci * (qsq - H);
  LV[3][1] = u * gm * ci;
  LV[3][2] = v * gm * ci;
  LV[3][3] = ww * gm * ci;
  LV[3][4] = -gm * ci;
  LV[4][0] = -0.5 * ci * (u - 0.5 * gm * qsq);
  LV[4][1] = -0.5 * ci * (gm * u - 1.0);
  LV[4][2] = -0.5 * v * gm * ci;
  LV[4][3] = -0.5 * ww * gm * ci;
  LV[4][4] = 0.5 * gm * ci;

  /* point fluxes and the Lax-Friedrichs speed */
  double alpha = 0.0;
  for (int j = 0; j < STS; ++j) {
    const double uj = W(j, 1) / W(j, 0);
    flux[j][0] = W(j, 1);
    flux[j][1] = uj * W(j, 1) + p[j];
    flux[j][2] = uj * W(j, 2);
    flux[j][3] = uj * W(j, 3);
    flux[j][4] = uj * (W(j, 4) + p[j]);
    for (int i = 5; i < nv; ++i) flux[j][i] = uj * W(j, i);
    const double cj = rsqrt_or_zero(gamma * p[j] / W(j, 0));
    const double s = fabs(uj) + cj;
    alpha = (alpha < s) ? s : alpha;
  }

  for (int side = 0; side < 2; ++side) {
    /* side 0: f+ on points 0..4; side 1: f- on points 1..5 */
    for (int j = 0; j < STS - 1; ++j)
      for (int i = 0; i < nv; ++i)
        fs[j][i] = side == 0 ? 0.5 * (flux[j][i] + alpha * W(j, i))
                             : 0.5 * (flux[j + 1][i] - alpha * W(j + 1, i));
    for (int j = 0; j < STS - 1; ++j) {
      for (int i = 0; i < 5; ++i)
        fproj[j][i] = LV[i][0] * fs[j][0] + LV[i][1] * fs[j][1] + LV[i][2] * fs[j][2] +
                      LV[i][3] * fs[j][3] + LV[i][4] * fs[j][4];
      for (int i = 5; i < nv; ++i) fproj[j][i] = fs[j][i];
    }
    for (int i = 0; i < nv; ++i) {
      const double f0 = fproj[0][i], f1 = fproj[1][i], f2 = fproj[2][i], f3 = fproj[3][i],
                   f4 = fproj[4][i];
      const double b13 = 13.0 / 12.0, eps = 1e-6;
      double dA = f2 - 2.0 * f3 + f4, eA = 3.0 * f2 - 4.0 * f3 + f4;
      double dB = f1 - 2.0 * f2 + f3, eB = f1 - f3;
      double dC = f0 - 2.0 * f1 + f2, eC = f0 - 4.0 * f1 + 3.0 * f2;
      const double betaA = b13 * (dA * dA) + 0.25 * (eA * eA);
      const double betaB = b13 * (dB * dB) + 0.25 * (eB * eB);
      const double betaC = b13 * (dC * dC) + 0.25 * (eC * eC);
      double wA, wB, wC, qA, qB, qC;
      if (side == 0) {
        wA = 0.3 / ((eps + betaA) * (eps + betaA));
        wB = 0.6 / ((eps + betaB) * (eps + betaB));
        wC = 0.1 / ((eps + betaC) * (eps + betaC));
        qA = (1.0 / 3.0) * f2 + (5.0 / 6.0) * f3 - (1.0 / 6.0) * f4;
        qB = -(1.0 / 6.0) * f1 + (5.0 / 6.0) * f2 + (1.0 / 3.0) * f3;
        qC = (1.0 / 3.0) * f0 - (7.0 / 6.0) * f1 + (11.0 / 6.0) * f2;
        ff[i] = (qA * wA + qB * wB + qC * wC) / (wA + wB + wC);
      } else {
        wA = 0.1 / ((eps + betaA) * (eps + betaA));
        wB = 0.6 / ((eps + betaB) * (eps + betaB));
        wC = 0.3 / ((eps + betaC) * (eps + betaC));
        qA = (11.0 / 6.0) * f2 - (7.0 / 6.0) * f3 + (1.0 / 3.0) * f4;
        qB = (1.0 / 3.0) * f1 + (5.0 / 6.0) * f2 - (1.0 / 6.0) * f3;
        qC = -(1.0 / 6.0) * f0 + (5.0 / 6.0) * f1 + (1.0 / 3.0) * f2;
        ff[i] += (qA * wA + qB * wB + qC * wC) / (wA + wB + wC);
      }
    }
  }

  for (int i = 0; i < 5; ++i)
    f_face[i] = RV[i][0] * ff[0] + RV[i][1] * ff[1] + RV[i][2] * ff[2] + RV[i][3] * ff[3] +
                RV[i][4] * ff[4];
  for (int i = 5; i < nv; ++i) f_face[i] = ff[i];
  if (idir > 0) {
    double t = f_face[1];
    f_face[1] = f_face[1 + idir];
    f_face[1 + idir] = t;
  }
#undef W
}

/* fEuler (src/utilities.cpp:17-253): forcing, all lower faces plus the upper boundary faces,
 * then wdot = G - [(Fx(i+1)-Fx(i))/dx + (Fy(j+1)-Fy(j))/dy + (Fz(k+1)-Fz(k))/dz].
 * This form evaluates the output planes k0 <= k < k1 only (the x and y faces of those planes
 * and the z faces k0 .. k1), reading the whole input; each output value is computed exactly as
 * in the whole-grid evaluation, so disjoint slabs can run on separate threads.  The legal-state
 * test covers the slab's cells (the whole grid's status is the OR over the slabs). */
int orc_feuler_slab(const orc_grid* g, const double* const* w, double* const* wdot,
                    const double* force, long k0, long k1) {
  const long nx = g->nx, ny = g->ny, nz = g->nz;
  const int nv = 5 + g->nchem;
  if (k0 < 0) k0 = 0;
  if (k1 > nz) k1 = nz;
  if (k1 <= k0) return 0;
  const long nk = k1 - k0;
  for (long c = k0 * nx * ny; c < k1 * nx * ny; ++c)
    if (legal_state(g->gamma, w[0][c], w[1][c], w[2][c], w[3][c], w[4][c])) return -1;

  double* fl[3];
  /* face extents of the slab; face (i, j, kk) of direction d has global plane k0 + kk */
  const long fext[3][3] = {{nx + 1, ny, nk}, {nx, ny + 1, nk}, {nx, ny, nk + 1}};
  for (int d = 0; d < 3; ++d)
    fl[d] = (double*)malloc(sizeof(double) * nv * fext[d][0] * fext[d][1] * fext[d][2]);
  double w1d[STS * MAXVAR];
  for (int d = 0; d < 3; ++d) {
    const long ex = fext[d][0], ey = fext[d][1], ez = fext[d][2];
    for (long kk = 0; kk < ez; ++kk)
      for (long j = 0; j < ey; ++j)
        for (long i = 0; i < ex; ++i) {
          for (int l = 0; l < STS; ++l) {
            long p[3] = {i, j, k0 + kk};
            p[d] += l - 3;
            for (int v = 0; v < nv; ++v) w1d[l * nv + v] = field_at(g, w, v, p);
          }
          orc_face_flux(g, w1d, d, &fl[d][nv * (i + ex * (j + ey * kk))]);
        }
  }
  const double dd[3] = {g->dx, g->dy, g->dz};
  for (long kk = 0; kk < nk; ++kk)
    for (long j = 0; j < ny; ++j)
      for (long i = 0; i < nx; ++i) {
        const long c = i + nx * (j + ny * (k0 + kk));
        const long lo[3] = {nv * (i + (nx + 1) * (j + ny * kk)), nv * (i + nx * (j + (ny + 1) * kk)),
                            nv * (i + nx * (j + ny * kk))};
        const long hi[3] = {lo[0] + nv, lo[1] + nv * nx, lo[2] + nv * nx * ny};
        for (int v = 0; v < nv; ++v) {
          const double div = (fl[0][hi[0] + v] - fl[0][lo[0] + v]) / dd[0] +
                             (fl[1][hi[1] + v] - fl[1][lo[1] + v]) / dd[1] +
                             (fl[2][hi[2] + v] - fl[2][lo[2] + v]) / dd[2];
          const double G = force ? force[v] : 0.0;
          if (v < 5)
            wdot[v][c] = G - div;
          else
            wdot[5][(v - 5) + (long)g->nchem * c] = G - div;
        }
      }
  for (int d = 0; d < 3; ++d) free(fl[d]);
  return 0;
}

int orc_feuler(const orc_grid* g, const double* const* w, double* const* wdot,
               const double* force) {
  /* the whole grid's legal-state test comes first: nothing is written for an illegal state */
  const long n = g->nx * g->ny * g->nz;
  for (long c = 0; c < n; ++c)
    if (legal_state(g->gamma, w[0][c], w[1][c], w[2][c], w[3][c], w[4][c])) return -1;
  return orc_feuler_slab(g, w, wdot, force, 0, g->nz);
}

/* -------------------------------------------------------------- chemistry */

/* Table rows (order of h5tables.TABLE_NAMES). */
enum {
  T_K01, T_K02, T_K03, T_K04, T_K05, T_K06, T_K07, T_K08, T_K09, T_K10, T_K11, T_K12, T_K13,
  T_K14, T_K15, T_K16, T_K17, T_K18, T_K19, T_K21, T_K22,
  T_BREM, T_CEHEI, T_CEHEII, T_CEHI, T_CIECO, T_CIHEI, T_CIHEII, T_CIHEIS, T_CIHI, T_COMPTON,
  T_GAEL, T_GAH2, T_GAHE, T_GAHI, T_GAHP, T_H2LTE, T_H2MCOOL, T_H2MHEAT, T_NCRD1, T_NCRD2,
  T_NCRN, T_REHEII1, T_REHEII2, T_REHEIII, T_REHII,
  T_GAMMAH2_1, T_DGAMMAH2_1, T_GAMMAH2_2, T_DGAMMAH2_2, T_NUM
};
#define NRATES 46 /* rows T_K01 .. T_REHII are interpolated per cell */

void orc_chem_init(orc_chem* c, const double* tables, double z) {
  /* src/raja_primordial_network.cpp:190-194 */
  c->tables = tables;
  c->tlo = 1.0;
  c->thi = 100000.0;
  c->nbins = ORC_TSIZE - 1;
  c->lb = log(c->tlo);
  c->dbin = (log(c->thi) - log(c->tlo)) / c->nbins;
  c->idbin = (double)(1.0L / (long double)c->dbin);
  c->z = z;
}

static const double mH = 1.67e-24;

void orc_chem_aux(const double* scale, long n, double* mdens, double* imdens, double* cie_oda,
                  double* h2_oda) {
  /* src/raja_primordial_network.cpp:1969-2018 */
  static const double amu[8] = {2.0, 2.0, 1.00794, 1.00794, 1.00794, 4.002602, 4.002602, 4.002602};
  for (long i = 0; i < n; ++i) {
    double m = 0.0;
    for (int s = 0; s < 8; ++s) m += scale[i * 10 + s] * amu[s];
    m *= mH;
    double tau = pow(m / 3.3e-8, 2.8);
    tau = fmax(tau, 1.0e-5);
    mdens[i] = m;
    imdens[i] = 1.0 / m;
    cie_oda[i] = fmin(1.0, (1.0 - exp(-tau)) / tau);
    h2_oda[i] = fmin(1.0, pow(m / 1.34e-14, -0.45));
  }
}

/* Bin lookup shared by the temperature solve and the rate interpolation
 * (src/raja_primordial_network.cpp:946-957, 1046-1061). */
static int lookup_bin(const orc_chem* c, double logT, double* t1, double* t2) {
  int b = (int)(c->idbin * (logT - c->lb));
  if (b <= 0) b = 0;
  else if (b >= c->nbins) b = c->nbins - 1;
  *t1 = c->lb + b * c->dbin;
  *t2 = c->lb + (b + 1) * c->dbin;
  return b;
}

static double lerp_row(const orc_chem* c, int row, int b, double Tdef) {
  const double* r = c->tables + (long)row * ORC_TSIZE;
  return r[b] + Tdef * (r[b + 1] - r[b]);
}

/* cvklu_calculate_temperature (src/raja_primordial_network.cpp:908-1011): exactly ten Newton
 * iterations on T(ge) with the H2 adiabatic indices interpolated in log T, starting from the
 * previous call's T; clamp to the table range afterwards; dT/dge from the last iteration. */
static void temperature(const orc_chem* c, const double* y, double* Ts, double* dTs_ge) {
  const double kb = 1.3806504e-16, gamma = 5.e0 / 3.e0, gm1 = 1.0 / (gamma - 1);
  const double H2_1 = y[0], H2_2 = y[1], H_1 = y[2], H_2 = y[3], H_m0 = y[4], He_1 = y[5],
               He_2 = y[6], He_3 = y[7], de = y[8], ge = y[9];
  const double density = 2.0 * H2_1 + 2.0 * H2_2 + 1.00794 * H_1 + 1.00794 * H_2 +
                         1.00794 * H_m0 + 4.002602 * He_1 + 4.002602 * He_2 + 4.002602 * He_3;
  double T, Tnew = 0.0, dge_dT = 0.0;
  for (int it = 0; it < 10; ++it) {
    T = *Ts;
    double t1, t2;
    const double logT = log(*Ts);
    const int b = lookup_bin(c, logT, &t1, &t2);
    const double Tdef = (log(*Ts) - t1) / (t2 - t1);
    const double g2 = lerp_row(c, T_GAMMAH2_2, b, Tdef);
    const double dg2 = lerp_row(c, T_DGAMMAH2_2, b, Tdef);
    const double g1 = lerp_row(c, T_GAMMAH2_1, b, Tdef);
    const double dg1 = lerp_row(c, T_DGAMMAH2_1, b, Tdef);
    const double i1 = 1.0 / (g1 - 1.0), i2 = 1.0 / (g2 - 1.0);
    const double nsum = H2_1 * i1 + H2_2 * i2 + H_1 * gm1 + H_2 * gm1 + H_m0 * gm1 + He_1 * gm1 +
                        He_2 * gm1 + He_3 * gm1 + gm1 * de;
    dge_dT = T * kb * (-H2_1 * i1 * i1 * dg1 - H2_2 * i2 * i2 * dg2) / (density * mH) +
             kb * nsum / (density * mH);
    const double dge = T * kb * nsum / (density * mH) - ge;
    Tnew = T - dge / dge_dT;
    *Ts = Tnew;
  }
  *Ts = Tnew;
  if (*Ts < c->tlo) *Ts = c->tlo;
  else if (*Ts > c->thi) *Ts = c->thi;
  *dTs_ge = 1.0 / dge_dT;
}

/* Per-cell rates k(T) and slopes dk/dT at the temperature Ts
 * (src/raja_primordial_network.cpp:1044-1248). */
static void rates_at(const orc_chem* c, double Ts, double* k, double* dk) {
  double t1, t2;
  const double logT = log(Ts);
  const int b = lookup_bin(c, logT, &t1, &t2);
  const double Tdef = (log(Ts) - t1) / (t2 - t1);
  const double dT = t2 - t1;
  const double invTs = 1.0 / Ts;
  const double Tfactor = invTs / dT;
  for (int r = 0; r < NRATES; ++r) {
    const double* row = c->tables + (long)r * ORC_TSIZE;
    k[r] = row[b] + Tdef * (row[b + 1] - row[b]);
    dk[r] = (row[b + 1] - row[b]) * Tfactor;
  }
}

/* Reaction fluxes r_m = k_m * (reactant product), m over the 21 reactions, factor order as
 * in the reference's expressions (src/raja_primordial_network.cpp:1305-1366). */
static void reaction_fluxes(const double* k, const double* y, double* r) {
  const double H2_1 = y[0], H2_2 = y[1], H_1 = y[2], H_2 = y[3], H_m0 = y[4], He_1 = y[5],
               He_2 = y[6], He_3 = y[7], de = y[8];
  r[0] = k[T_K01] * H_1 * de;
  r[1] = k[T_K02] * H_2 * de;
  r[2] = k[T_K03] * He_1 * de;
  r[3] = k[T_K04] * He_2 * de;
  r[4] = k[T_K05] * He_2 * de;
  r[5] = k[T_K06] * He_3 * de;
  r[6] = k[T_K07] * H_1 * de;
  r[7] = k[T_K08] * H_1 * H_m0;
  r[8] = k[T_K09] * H_1 * H_2;
  r[9] = k[T_K10] * H2_2 * H_1;
  r[10] = k[T_K11] * H2_1 * H_2;
  r[11] = k[T_K12] * H2_1 * de;
  r[12] = k[T_K13] * H2_1 * H_1;
  r[13] = k[T_K14] * H_m0 * de;
  r[14] = k[T_K15] * H_1 * H_m0;
  r[15] = k[T_K16] * H_2 * H_m0;
  r[16] = k[T_K17] * H_2 * H_m0;
  r[17] = k[T_K18] * H2_2 * de;
  r[18] = k[T_K19] * H2_2 * H_m0;
  r[19] = k[T_K21] * H2_1 * H_1 * H_1;
  r[20] = k[T_K22] * H_1 * H_1 * H_1;
}

/* Net stoichiometry of the nine species rows (src/raja_primordial_network.cpp:1305-1366),
 * listed in reaction order: {reaction index, coefficient}, terminated by {-1, 0}. */
static const int STOICH[9][17][2] = {
    /* H2_1 */ {{7, 1}, {9, 1}, {10, -1}, {11, -1}, {12, -1}, {18, 1}, {19, 1}, {20, 1}, {-1, 0}},
    /* H2_2 */ {{8, 1}, {9, -1}, {10, 1}, {16, 1}, {17, -1}, {18, -1}, {-1, 0}},
    /* H_1  */ {{0, -1}, {1, 1}, {6, -1}, {7, -1}, {8, -1}, {9, -1}, {10, 1}, {11, 2}, {12, 2},
                {13, 1}, {14, 1}, {15, 2}, {17, 2}, {18, 1}, {19, -2}, {20, -2}, {-1, 0}},
    /* H_2  */ {{0, 1}, {1, -1}, {8, -1}, {9, 1}, {10, -1}, {15, -1}, {16, -1}, {-1, 0}},
    /* H_m0 */ {{6, 1}, {7, -1}, {13, -1}, {14, -1}, {15, -1}, {16, -1}, {18, -1}, {-1, 0}},
    /* He_1 */ {{2, -1}, {3, 1}, {-1, 0}},
    /* He_2 */ {{2, 1}, {3, -1}, {4, -1}, {5, 1}, {-1, 0}},
    /* He_3 */ {{4, 1}, {5, -1}, {-1, 0}},
    /* de   */ {{0, 1}, {1, -1}, {2, 1}, {3, -1}, {4, 1}, {5, -1}, {6, -1}, {7, 1}, {13, 1},
                {14, 1}, {16, 1}, {17, -1}, {-1, 0}},
};

static double species_sum(int s, const double* r) {
  double acc = 0.0;
  for (int t = 0; STOICH[s][t][0] >= 0; ++t) {
    const double term = STOICH[s][t][1] * r[STOICH[s][t][0]];
    acc = (t == 0) ? term : acc + term;
  }
  return acc;
}

/* Gas-energy source term (src/raja_primordial_network.cpp:1371-1375): cooling/heating with
 * the optical-depth factors frozen at setup. */
static double ge_source(const orc_chem* c, const double* k, const double* y, double T,
                        double mdens, double cie, double h2oda) {
  const double H2_1 = y[0], H_1 = y[2], H_2 = y[3], He_1 = y[5], He_2 = y[6], He_3 = y[7],
               de = y[8];
  const double z = c->z;
  const double G = H2_1 * k[T_GAH2] + H_1 * k[T_GAHI] + H_2 * k[T_GAHP] + He_1 * k[T_GAHE] +
                   de * k[T_GAEL];
  const double D = k[T_H2LTE] / G + 1.0;
  const double F = k[T_NCRN] / (H2_1 * k[T_NCRD2] + H_1 * k[T_NCRD1]) + 1.0;
  const double Hf = -H2_1 * H_1 * k[T_H2MCOOL] + pow(H_1, 3) * k[T_H2MHEAT];
  return -2.01588 * H2_1 * k[T_CIECO] * cie * mdens - H2_1 * cie * k[T_H2LTE] * h2oda / D -
         H_1 * k[T_CEHI] * cie * de - H_1 * k[T_CIHI] * cie * de - H_2 * cie * de * k[T_REHII] -
         He_1 * k[T_CIHEI] * cie * de - He_2 * k[T_CEHEII] * cie * de -
         He_2 * k[T_CEHEI] * cie * pow(de, 2) - He_2 * k[T_CIHEII] * cie * de -
         He_2 * k[T_CIHEIS] * cie * pow(de, 2) - He_2 * cie * de * k[T_REHEII1] -
         He_2 * cie * de * k[T_REHEII2] - He_3 * cie * de * k[T_REHEIII] -
         k[T_BREM] * cie * de * (H_2 + He_2 + 4.0 * He_3) -
         cie * k[T_COMPTON] * de * pow(z + 1.0, 4) * (T - 2.73 * z - 2.73) +
         0.5 * 1.0 / F * Hf;
}

void orc_chem_rhs(const orc_chem* c, long n, const double* y, const double* scale,
                  const double* inv_scale, const double* mdens, const double* imdens,
                  const double* cie_oda, const double* h2_oda, double* Ts, double* dTs_ge,
                  double* ydot) {
  for (long i = 0; i < n; ++i) {
    const long j = i * 10;
    double ya[10], k[NRATES], dk[NRATES], r[21];
    for (int s = 0; s < 10; ++s) ya[s] = y[j + s] * scale[j + s];
    temperature(c, ya, &Ts[i], &dTs_ge[i]);
    rates_at(c, Ts[i], k, dk);
    reaction_fluxes(k, ya, r);
    for (int s = 0; s < 9; ++s) {
      ydot[j + s] = species_sum(s, r);
      ydot[j + s] *= inv_scale[j + s];
    }
    ydot[j + 9] = ge_source(c, k, ya, Ts[i], mdens[i], cie_oda[i], h2_oda[i]);
    ydot[j + 9] *= inv_scale[j + 9];
    ydot[j + 9] *= imdens[i];
  }
}

void orc_chem_jac(const orc_chem* c, long n, const double* y, const double* scale,
                  const double* inv_scale, const double* mdens, const double* cie_oda,
                  const double* h2_oda, const double* Ts, const double* dTs_ge, double* J) {
  (void)cie_oda;
  for (long i = 0; i < n; ++i) {
    const long j = i * 10;
    double ya[10], k[NRATES], dk[NRATES], r[21];
    for (int s = 0; s < 10; ++s) ya[s] = y[j + s] * scale[j + s];
    const double H2_1 = ya[0], H2_2 = ya[1], H_1 = ya[2], H_2 = ya[3], H_m0 = ya[4],
                 He_1 = ya[5], He_2 = ya[6], He_3 = ya[7], de = ya[8];
    const double T = Ts[i], Tge = dTs_ge[i], z = c->z;
    const double md = mdens[i], imd = 1.0 / md, h2oda = h2_oda[i];
    rates_at(c, T, k, dk);
    double* B = J + 100 * i;
    for (int e = 0; e < 100; ++e) B[e] = 0.0;
#define K(x) k[T_##x]
#define R(x) dk[T_##x]
#define SET(row, col, expr) B[(col) * 10 + (row)] = (expr)
    /* src/raja_primordial_network.cpp:1518-1815, species rows by species columns */
    SET(0, 0, -K(K11) * H_2 - K(K12) * de - K(K13) * H_1 + K(K21) * pow(H_1, 2));
    SET(0, 1, K(K10) * H_1 + K(K19) * H_m0);
    SET(0, 2, K(K08) * H_m0 + K(K10) * H2_2 - K(K13) * H2_1 + 2 * K(K21) * H2_1 * H_1 +
                  3 * K(K22) * pow(H_1, 2));
    SET(0, 3, -K(K11) * H2_1);
    SET(0, 4, K(K08) * H_1 + K(K19) * H2_2);
    SET(0, 8, -K(K12) * H2_1);
    SET(1, 0, K(K11) * H_2);
    SET(1, 1, -K(K10) * H_1 - K(K18) * de - K(K19) * H_m0);
    SET(1, 2, K(K09) * H_2 - K(K10) * H2_2);
    SET(1, 3, K(K09) * H_1 + K(K11) * H2_1 + K(K17) * H_m0);
    SET(1, 4, K(K17) * H_2 - K(K19) * H2_2);
    SET(1, 8, -K(K18) * H2_2);
    SET(2, 0, K(K11) * H_2 + 2 * K(K12) * de + 2 * K(K13) * H_1 - 2 * K(K21) * pow(H_1, 2));
    SET(2, 1, -K(K10) * H_1 + 2 * K(K18) * de + K(K19) * H_m0);
    SET(2, 2, -K(K01) * de - K(K07) * de - K(K08) * H_m0 - K(K09) * H_2 - K(K10) * H2_2 +
                  2 * K(K13) * H2_1 + K(K15) * H_m0 - 4 * K(K21) * H2_1 * H_1 -
                  6 * K(K22) * pow(H_1, 2));
    SET(2, 3, K(K02) * de - K(K09) * H_1 + K(K11) * H2_1 + 2 * K(K16) * H_m0);
    SET(2, 4, -K(K08) * H_1 + K(K14) * de + K(K15) * H_1 + 2 * K(K16) * H_2 + K(K19) * H2_2);
    SET(2, 8, -K(K01) * H_1 + K(K02) * H_2 - K(K07) * H_1 + 2 * K(K12) * H2_1 +
                  K(K14) * H_m0 + 2 * K(K18) * H2_2);
    SET(3, 0, -K(K11) * H_2);
    SET(3, 1, K(K10) * H_1);
    SET(3, 2, K(K01) * de - K(K09) * H_2 + K(K10) * H2_2);
    SET(3, 3, -K(K02) * de - K(K09) * H_1 - K(K11) * H2_1 - K(K16) * H_m0 - K(K17) * H_m0);
    SET(3, 4, -K(K16) * H_2 - K(K17) * H_2);
    SET(3, 8, K(K01) * H_1 - K(K02) * H_2);
    SET(4, 1, -K(K19) * H_m0);
    SET(4, 2, K(K07) * de - K(K08) * H_m0 - K(K15) * H_m0);
    SET(4, 3, -K(K16) * H_m0 - K(K17) * H_m0);
    SET(4, 4, -K(K08) * H_1 - K(K14) * de - K(K15) * H_1 - K(K16) * H_2 - K(K17) * H_2 -
                  K(K19) * H2_2);
    SET(4, 8, K(K07) * H_1 - K(K14) * H_m0);
    SET(5, 5, -K(K03) * de);
    SET(5, 6, K(K04) * de);
    SET(5, 8, -K(K03) * He_1 + K(K04) * He_2);
    SET(6, 5, K(K03) * de);
    SET(6, 6, -K(K04) * de - K(K05) * de);
    SET(6, 7, K(K06) * de);
    SET(6, 8, K(K03) * He_1 - K(K04) * He_2 - K(K05) * He_2 + K(K06) * He_3);
    SET(7, 6, K(K05) * de);
    SET(7, 7, -K(K06) * de);
    SET(7, 8, K(K05) * He_2 - K(K06) * He_3);
    SET(8, 1, -K(K18) * de);
    SET(8, 2, K(K01) * de - K(K07) * de + K(K08) * H_m0 + K(K15) * H_m0);
    SET(8, 3, -K(K02) * de + K(K17) * H_m0);
    SET(8, 4, K(K08) * H_1 + K(K14) * de + K(K15) * H_1 + K(K17) * H_2);
    SET(8, 5, K(K03) * de);
    SET(8, 6, -K(K04) * de + K(K05) * de);
    SET(8, 7, -K(K06) * de);
    SET(8, 8, K(K01) * H_1 - K(K02) * H_2 + K(K03) * He_1 - K(K04) * He_2 + K(K05) * He_2 -
                  K(K06) * He_3 - K(K07) * H_1 + K(K14) * H_m0 - K(K18) * H2_2);
    /* species rows by ge: the species source with rates replaced by their T slopes, times
     * dT/dge (src/raja_primordial_network.cpp:1546-1788, "by ge" entries) */
    reaction_fluxes(dk, ya, r);
    for (int s = 0; s < 9; ++s) {
      SET(s, 9, species_sum(s, r));
      B[90 + s] *= Tge;
    }
    /* ge row (src/raja_primordial_network.cpp:1793-1860) */
    const double G = H2_1 * K(GAH2) + H_1 * K(GAHI) + H_2 * K(GAHP) + He_1 * K(GAHE) +
                     de * K(GAEL);
    const double D = K(H2LTE) / G + 1.0;
    const double N = H2_1 * K(NCRD2) + H_1 * K(NCRD1);
    const double F = K(NCRN) / N + 1.0;
    const double Hf = -H2_1 * H_1 * K(H2MCOOL) + pow(H_1, 3) * K(H2MHEAT);
    const double lte2 = pow(K(H2LTE), 2);
    const double DG2 = pow(D, 2) * pow(G, 2);
    SET(9, 0, -H2_1 * K(GAH2) * lte2 * h2oda / DG2 - 0.5 * H_1 * K(H2MCOOL) * 1.0 / F -
                  2.01588 * K(CIECO) * md - K(H2LTE) * h2oda / D +
                  0.5 * K(NCRD2) * K(NCRN) * pow(F, -2.0) * Hf / pow(N, 2));
    SET(9, 2, -H2_1 * K(GAHI) * lte2 * h2oda / DG2 - K(CEHI) * de - K(CIHI) * de +
                  0.5 * K(NCRD1) * K(NCRN) * pow(F, -2.0) * Hf / pow(N, 2) +
                  0.5 * (-H2_1 * K(H2MCOOL) + 3 * pow(H_1, 2) * K(H2MHEAT)) * 1.0 / F);
    SET(9, 3, -H2_1 * K(GAHP) * lte2 * h2oda / DG2 - K(BREM) * de - de * K(REHII));
    SET(9, 5, -H2_1 * K(GAHE) * lte2 * h2oda / DG2 - K(CIHEI) * de);
    SET(9, 6, -K(BREM) * de - K(CEHEII) * de - K(CEHEI) * pow(de, 2) - K(CIHEII) * de -
                  K(CIHEIS) * pow(de, 2) - de * K(REHEII1) - de * K(REHEII2));
    SET(9, 7, -4.0 * K(BREM) * de - de * K(REHEIII));
    SET(9, 8, -H2_1 * K(GAEL) * lte2 * h2oda / DG2 - H_1 * K(CEHI) - H_1 * K(CIHI) -
                  H_2 * K(REHII) - He_1 * K(CIHEI) - He_2 * K(CEHEII) -
                  2 * He_2 * K(CEHEI) * de - He_2 * K(CIHEII) - 2 * He_2 * K(CIHEIS) * de -
                  He_2 * K(REHEII1) - He_2 * K(REHEII2) - He_3 * K(REHEIII) -
                  K(BREM) * (H_2 + He_2 + 4.0 * He_3) -
                  K(COMPTON) * pow(z + 1.0, 4) * (T - 2.73 * z - 2.73));
    /* the reference's "ad-hoc" ge-by-ge entry (h2 formation and line cooling only) */
    const double dGn = -H2_1 * R(GAH2) - H_1 * R(GAHI) - H_2 * R(GAHP) - He_1 * R(GAHE) -
                       de * R(GAEL);
    SET(9, 9, -H2_1 * K(H2LTE) * h2oda * (-K(H2LTE) * dGn / pow(G, 2) - R(H2LTE) / G) /
                      pow(D, 2) -
                  H2_1 * h2oda * R(H2LTE) / D +
                  0.5 * pow(F, -2.0) * Hf *
                      (-1.0 * K(NCRN) * (-H2_1 * R(NCRD2) - H_1 * R(NCRD1)) / pow(N, 2) -
                       1.0 * R(NCRN) / N) +
                  0.5 * 1.0 / F * (-H2_1 * H_1 * R(H2MCOOL) + pow(H_1, 3) * R(H2MHEAT)));
    for (int col = 0; col < 10; ++col) B[col * 10 + 9] *= imd;
    B[99] *= Tge;
    /* unit scaling of every nonzero (src/raja_primordial_network.cpp: "*= inv_scale*scale") */
    for (int col = 0; col < 10; ++col)
      for (int row = 0; row < 10; ++row) B[col * 10 + row] *= (inv_scale[j + row] * scale[j + col]);
#undef K
#undef R
#undef SET
  }
}

/* Dense LU with partial pivoting on one column-major 10x10 block (the algorithm of LAPACK
 * dgetrf/dgetrs, as used by the reference's SUNLinSol_MagmaDense / batched getrf). */
static int lu10(double* A, int* piv) {
  int info = 0;
  for (int kk = 0; kk < 10; ++kk) {
    int p = kk;
    double amax = fabs(A[kk * 10 + kk]);
    for (int r = kk + 1; r < 10; ++r)
      if (fabs(A[kk * 10 + r]) > amax) { amax = fabs(A[kk * 10 + r]); p = r; }
    piv[kk] = p;
    if (A[kk * 10 + p] == 0.0) { if (!info) info = kk + 1; continue; }
    if (p != kk)
      for (int col = 0; col < 10; ++col) {
        double t = A[col * 10 + kk];
        A[col * 10 + kk] = A[col * 10 + p];
        A[col * 10 + p] = t;
      }
    const double rp = 1.0 / A[kk * 10 + kk];
    for (int r = kk + 1; r < 10; ++r) A[kk * 10 + r] *= rp;
    for (int col = kk + 1; col < 10; ++col) {
      const double a = A[col * 10 + kk];
      for (int r = kk + 1; r < 10; ++r) A[col * 10 + r] -= A[kk * 10 + r] * a;
    }
  }
  return info;
}

static void lus10(const double* A, const int* piv, double* x) {
  for (int kk = 0; kk < 10; ++kk)
    if (piv[kk] != kk) { double t = x[kk]; x[kk] = x[piv[kk]]; x[piv[kk]] = t; }
  for (int col = 0; col < 10; ++col)
    for (int r = col + 1; r < 10; ++r) x[r] -= A[col * 10 + r] * x[col];
  for (int col = 9; col >= 0; --col) {
    x[col] /= A[col * 10 + col];
    for (int r = 0; r < col; ++r) x[r] -= A[col * 10 + r] * x[col];
  }
}

long orc_block_newton_solve(long n, const double* J, double gamma, const double* b, double* x) {
  long first_bad = 0;
  for (long i = 0; i < n; ++i) {
    double A[100];
    int piv[10];
    for (int col = 0; col < 10; ++col)
      for (int r = 0; r < 10; ++r)
        A[col * 10 + r] = -gamma * J[100 * i + col * 10 + r] + (r == col ? 1.0 : 0.0);
    for (int s = 0; s < 10; ++s) x[10 * i + s] = b[10 * i + s];
    if (lu10(A, piv)) {
      if (!first_bad) first_bad = i + 1;
      continue;
    }
    lus10(A, piv, &x[10 * i]);
  }
  return first_bad;
}

/* ------------------------------------------------------------------------------------------
 * Per-cell adaptive DIRK integration of the scaled chemistry system dz/dt = tunit * f(z):
 * the CPU restatement of the persistent GPU integrator (gbmv_chem_dirk_evolve), FP64
 * throughout.  The reference integrates the same system with ARKStep (DIRK + Newton +
 * block-diagonal direct solver, src/primordial_ode_main.cpp) over all cells at once; this
 * restatement applies ARKODE's Newton and step rules per cell (see oracle.h), except that no
 * Jacobian is kept between Newton-matrix setups (each setup evaluates J at the step's state)
 * and the WRMS weights are rounded to float, as the GPU kernel stores them.
 * The method is the stiffly accurate ESDIRK given in O (ARK4(3)7L[2]SA's implicit part, the
 * reference inputs' itable 112, or TR-BDF2, itable 102): stage i of s solves
 * z_i = y + h sum_{j<i} a_ij K_j + h gamma F(z_i) from the previous stage's value, y_{n+1} =
 * z_s, and h sum_j e_j K_j (e = b - bhat) is the embedded error estimate of order p. */

/* safety dsm^(-1/p) */
static double dk_eta(double safety, double dsm, int p) {
  if (p == 3) return safety / cbrt(dsm);
  if (p == 2) return safety / sqrt(dsm);
  return safety * pow(dsm, -1.0 / p);
}

static void dirk_F(const orc_chem* c, const double* X, const double* sc, const double* isc,
                   double md, double imd, double cie, double h2, const orc_dirk_opts* O,
                   long cell, double tf, double* Ts, double* dTs, double* f) {
  const double tunit = O->tunit;
  double ya[10], k[NRATES], dk[NRATES], r[21];
  for (int s = 0; s < 10; ++s) ya[s] = X[s] * sc[s];
  temperature(c, ya, Ts, dTs);
  rates_at(c, *Ts, k, dk);
  reaction_fluxes(k, ya, r);
  for (int s = 0; s < 9; ++s) f[s] = (species_sum(s, r) * isc[s]) * tunit;
  double ge = ge_source(c, k, ya, *Ts, md, cie, h2) * isc[9];
  ge *= imd;
  f[9] = ge * tunit;
  if (O->nforcing > 0) {
    const double tau = (tf - O->tshift) / O->tscale;
    double p = 1.0;
    for (int q = 0; q < O->nforcing; ++q) {
      for (int s = 0; s < 10; ++s) f[s] += p * O->fz[q][cell * 10 + s];
      p *= tau;
    }
  }
}

static double dk_wrms(const double* v, const double* ew) {
  double s2 = 0.0;
  for (int s = 0; s < 10; ++s) {
    const double q = v[s] * ew[s];
    s2 += q * q;
  }
  return sqrt(s2 / 10.0);
}

long orc_chem_dirk_evolve(const orc_chem* c, long n, double* y, const double* scale,
                          const double* inv_scale, const double* mdens, const double* imdens,
                          const double* cie_oda, const double* h2_oda, double* Ts, double* dTs_ge,
                          const orc_dirk_opts* O, int* stats) {
  const int ns = O->s;
  long nfail = 0;
  for (long i = 0; i < n; ++i) {
    const long j = i * 10;
    const double *sc = scale + j, *isc = inv_scale + j;
    const double md = mdens[i], imd = imdens[i], cie = cie_oda[i], h2 = h2_oda[i];
    double Y[10], K1[10], KS[7][10], Z[10], EW[10], f[10], A[100];
    int piv[10];
    for (int s = 0; s < 10; ++s) Y[s] = y[j + s];
    double Tsc = Ts[i], dTsc = dTs_ge[i], Tsy, dTsy;
    double t = O->t0, h = O->h0, gp = 0.0, crate = 1.0, delp = 0.0;
    int nst = 0, nst_lp = 0, nef_s = 0, ncf_s = 0;
    int nni = 0, netf = 0, ncf = 0, nsetup = 0, nfe = 0;
    int jcur = 0, force_setup = 1, last = 0, failed = 0;
    dirk_F(c, Y, sc, isc, md, imd, cie, h2, O, i, t, &Tsc, &dTsc, K1);
    ++nfe;
    Tsy = Tsc;
    dTsy = dTsc;
    if (h <= 0.0) {
      double s2 = 0.0;
      for (int s = 0; s < 10; ++s) {
        const double v = K1[s] / (O->rtol * fabs(Y[s]) + O->atol);
        s2 += v * v;
      }
      const double fn = sqrt(s2 / 10.0);
      h = (fn > 0.0) ? O->h0fac / fn : O->tout - t;
    }
    if (O->hmax > 0.0 && h > O->hmax) h = O->hmax;
    for (;;) {
      /* step setup: weights, predictor, Jacobian / Newton matrix as needed */
      for (;;) {
        last = (t + h >= O->tout);
        if (last) h = O->tout - t;
        Tsc = Tsy;
        dTsc = dTsy;
        for (int s = 0; s < 10; ++s) {
          EW[s] = (double)(float)(1.0 / (O->rtol * fabs(Y[s]) + O->atol)); /* float weights */
          Z[s] = Y[s];
        }
        const double gam = h * O->gamma;
        if (force_setup || nst >= nst_lp + O->msbp || !(fabs(gam / gp - 1.0) <= O->dgmax)) {
          /* no Jacobian is kept between setups: J at (Y, Ts(Y)) for every Newton matrix */
          double B[100];
          orc_chem_jac(c, 1, Y, sc, isc, &mdens[i], &cie_oda[i], &h2_oda[i], &Tsy, &dTsy, B);
          const double mg = -gam * O->tunit;
          for (int col = 0; col < 10; ++col)
            for (int r = 0; r < 10; ++r)
              A[col * 10 + r] = (r == col ? 1.0 : 0.0) + mg * B[col * 10 + r];
          const int info = lu10(A, piv);
          gp = gam;
          nst_lp = nst;
          crate = 1.0;
          jcur = 1;
          force_setup = 0;
          ++nsetup;
          if (info) {
            ++ncf_s;
            ++ncf;
            if (ncf_s >= O->maxncf) { failed = 1; break; }
            h *= 0.25;
            force_setup = 1;
            continue;
          }
        }
        break;
      }
      if (failed) break;
      /* implicit stages 1 .. s-1 by modified Newton */
      int conv = 1;
      double tst = t;
      for (int st = 1; st < ns && conv; ++st) {
        const double gam = h * O->gamma;
        double Bv[10];
        const double c0 = h * O->a[st][0];
        for (int s = 0; s < 10; ++s) {
          Bv[s] = Y[s];
          if (c0 != 0.0) Bv[s] += c0 * K1[s];
        }
        for (int q = 1; q < st; ++q) {
          const double cq = h * O->a[st][q];
          if (cq == 0.0) continue;
          for (int s = 0; s < 10; ++s) Bv[s] += cq * KS[q][s];
        }
        tst = t + O->c[st] * h;
        int m = 0;
        conv = 0;
        for (;;) {
          dirk_F(c, Z, sc, isc, md, imd, cie, h2, O, i, tst, &Tsc, &dTsc, f);
          ++nfe;
          double dl[10];
          for (int s = 0; s < 10; ++s) dl[s] = Bv[s] + gam * f[s] - Z[s];
          lus10(A, piv, dl);
          if (gam != gp) {
            const double scl = 2.0 / (1.0 + gam / gp);
            for (int s = 0; s < 10; ++s) dl[s] *= scl;
          }
          for (int s = 0; s < 10; ++s) Z[s] += dl[s];
          const double del = dk_wrms(dl, EW);
          ++m;
          ++nni;
          if (m > 1) crate = fmax(0.3 * crate, del / delp);
          if (fmin(crate, 1.0) * del / O->nlscoef <= 1.0) { conv = 1; break; }
          if ((m > 1 && del > 2.3 * delp) || m >= O->maxcor || !(del == del)) break;
          delp = del;
        }
        if (conv && st < ns - 1) {
          if (O->deduce) { /* ARKODE's deduced implicit RHS: no F evaluation */
            const double rg = 1.0 / gam; /* as the GPU kernel: one reciprocal, ten products */
            for (int s = 0; s < 10; ++s) KS[st][s] = (Z[s] - Bv[s]) * rg;
          } else {
            dirk_F(c, Z, sc, isc, md, imd, cie, h2, O, i, tst, &Tsc, &dTsc, KS[st]);
            ++nfe;
          }
        }
      }
      if (!conv) {
        ++ncf_s;
        ++ncf;
        if (ncf_s >= O->maxncf) { failed = 1; break; }
        if (jcur) h *= 0.25;
        else force_setup = 1;
        continue;
      }
      dirk_F(c, Z, sc, isc, md, imd, cie, h2, O, i, tst, &Tsc, &dTsc, f);
      ++nfe;
      double err[10];
      for (int s = 0; s < 10; ++s) {
        double acc = O->e[0] * K1[s];
        for (int q = 1; q < ns - 1; ++q)
          if (O->e[q] != 0.0) acc += O->e[q] * KS[q][s];
        err[s] = h * (acc + O->e[ns - 1] * f[s]);
      }
      const double dsm = dk_wrms(err, EW);
      if (dsm <= 1.0) {
        ++nst;
        t = last ? O->tout : t + h;
        for (int s = 0; s < 10; ++s) {
          Y[s] = Z[s];
          K1[s] = f[s];
        }
        Tsy = Tsc;
        dTsy = dTsc;
        jcur = 0;
        double eta = (dsm > 0.0) ? dk_eta(O->safety, dsm, O->p) : 1.0e300;
        eta = fmin(eta, nst == 1 ? O->etamx1 : O->growth);
        if (nef_s > 0 || ncf_s > 0) eta = fmin(eta, 1.0);
        h *= eta;
        if (O->hmax > 0.0 && h > O->hmax) h = O->hmax;
        nef_s = ncf_s = 0;
        if (last) break;
        if (nst >= O->max_steps) { failed = 1; break; }
      } else {
        ++nef_s;
        ++netf;
        if (nef_s >= O->maxnef) { failed = 1; break; }
        double eta = fmax(0.1, dk_eta(O->safety, dsm, O->p));
        if (nef_s >= 2) eta = fmin(eta, 0.3);
        h *= eta;
      }
    }
    for (int s = 0; s < 10; ++s) y[j + s] = Y[s];
    Ts[i] = Tsy;
    dTs_ge[i] = dTsy;
    if (stats) {
      int* st = stats + i * 8;
      st[0] = nst; st[1] = nni; st[2] = netf; st[3] = ncf;
      st[4] = nsetup; st[5] = nsetup; st[6] = nfe; st[7] = failed;
    }
    nfail += failed;
  }
  return nfail;
}
