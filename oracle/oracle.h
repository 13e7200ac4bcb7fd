/* CPU oracle for the GB300 RHS hot path: a plain-C restatement of the reference's
 * algorithms, evaluated in the reference's operation order (compiled with
 * -ffp-contract=off so results match the reference's own CPU build to rounding).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference legs may load this library, and only as the checker or
 * as the timed CPU baseline; the product path never calls it.
 *
 * Pinned against the reference itself: oracle/build_ref.sh compiles the reference's
 * src/utilities.cpp, src/euler3D.hpp and src/raja_primordial_network.cpp unmodified, and
 * tests/golden/make_golden.py records their outputs; tests/test_oracle_golden.py checks this
 * restatement against those fixtures.
 */
#ifndef GBMV_ORACLE_H
#define GBMV_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NSPECIES 10
#define ORC_NTABLES 50
#define ORC_TSIZE 1024

/* Boundary-condition codes (src/euler3D.hpp:86-89). */
#define ORC_BC_PERIODIC 0
#define ORC_BC_NEUMANN 1
#define ORC_BC_DIRICHLET 2
#define ORC_BC_REFLECTING 3

typedef struct {
  long nx, ny, nz;   /* cells */
  int nchem;         /* advected species; NVAR = 5 + nchem */
  double dx, dy, dz; /* mesh spacing */
  double gamma;      /* ratio of specific heats */
  int bc[6];         /* x-lower, x-upper, y-lower, y-upper, z-lower, z-upper */
} orc_grid;

/* fEuler (src/utilities.cpp:17-253).  w: 5 SoA fluid arrays then the species-fastest
 * chemistry array (when nchem>0); wdot likewise.  force: NVAR per-field constants added as
 * the external forcing (NULL = 0).  Returns 0, or -1 if any cell is an illegal state
 * (src/euler3D.hpp:1405-1414). */
int orc_feuler(const orc_grid* g, const double* const* w, double* const* wdot,
               const double* force);

/* orc_feuler restricted to the output planes k0 <= k < k1 (reading the whole input): the same
 * values the whole-grid call writes there, so disjoint slabs may run on separate threads.
 * Returns -1 if a cell of the slab is an illegal state. */
int orc_feuler_slab(const orc_grid* g, const double* const* w, double* const* wdot,
                    const double* force, long k0, long k1);

/* face_flux on one 6-point stencil w1d[6][nvar] (src/utilities.cpp:270-479). */
void orc_face_flux(const orc_grid* g, double* w1d, int idir, double* f_face);

/* Chemistry network state shared by RHS and Jacobian. */
typedef struct {
  const double* tables;   /* [ORC_NTABLES][ORC_TSIZE], table order of h5tables.TABLE_NAMES */
  double dbin, idbin, lb; /* log-T bin width, its reciprocal, log(T lower bound) */
  int nbins;              /* ORC_TSIZE - 1 */
  double tlo, thi;        /* temperature bounds */
  double z;               /* redshift */
} orc_chem;

void orc_chem_init(orc_chem* c, const double* tables, double z);

/* setting_up_extra_variables (src/raja_primordial_network.cpp:1969-2018). */
void orc_chem_aux(const double* scale, long n, double* mdens, double* imdens, double* cie_oda,
                  double* h2_oda);

/* calculate_rhs_cvklu (src/raja_primordial_network.cpp:1015-1389).  Ts is read and updated
 * in place (the temperature Newton starts from the previous call's value); dTs_ge written. */
void orc_chem_rhs(const orc_chem* c, long n, const double* y, const double* scale,
                  const double* inv_scale, const double* mdens, const double* imdens,
                  const double* cie_oda, const double* h2_oda, double* Ts, double* dTs_ge,
                  double* ydot);

/* calculate_jacobian_cvklu (src/raja_primordial_network.cpp:1393-1965), dense column-major
 * 10x10 blocks J[i*100 + col*10 + row].  Uses the rates of the temperature Ts left by the
 * last RHS call. */
void orc_chem_jac(const orc_chem* c, long n, const double* y, const double* scale,
                  const double* inv_scale, const double* mdens, const double* cie_oda,
                  const double* h2_oda, const double* Ts, const double* dTs_ge, double* J);

/* Block-diagonal Newton solve: A_i = I - gamma*J_i (column-major 10x10), LU with partial
 * pivoting, then solve A_i x_i = b_i.  Returns 0 or (1 + first singular block index). */
long orc_block_newton_solve(long n, const double* J, double gamma, const double* b, double* x);

/* Options of orc_chem_dirk_evolve (the fields of gbmv_dirk_opts plus the resolved times). */
typedef struct {
  double t0, tout, tunit;
  double rtol, atol, nlscoef, h0, h0fac, safety, dgmax, growth, etamx1, hmax;
  int maxcor, max_steps, msbp, maxnef, maxncf;
  /* MRI forcing added to the right-hand side: sum_i tau^i fz[i] (10 values per cell),
   * tau = (t - tshift) / tscale (ffast, src/multirate_chem_hydro_main.cpp:921-944) */
  int nforcing;
  double tshift, tscale;
  const double* fz[8];
  /* the stiffly accurate ESDIRK: s stages, explicit first stage, diagonal gamma, stage i
   * solves z_i = y + h sum_{j<i} a[i][j] K_j + h gamma F(z_i); e = b - bhat, embedding
   * order p */
  int s, p;
  double gamma;
  double c[7];
  double a[7][7];
  double e[7];
  /* 1: the derivative of each converged intermediate stage from its stage equation,
   * K_i = (z_i - base_i) / (h gamma), instead of F(z_i) (gbmv_dirk_opts.deduce) */
  int deduce;
} orc_dirk_opts;

/* Per-cell adaptive ESDIRK integration (the table in O) of dz/dt = tunit * f_chem(z) (scaled
 * variables, as orc_chem_rhs x tunit) from t0 to tout, modified Newton with ARKODE's
 * convergence, reuse and step rules (a fresh J at every Newton-matrix setup), FP64 LU; the algorithm of the GPU integrator
 * (gbmv_chem_dirk_evolve).  y, Ts, dTs_ge updated in place; stats (8 ints per cell, or NULL):
 * steps, Newton iterations, error-test failures, Newton failures, matrix setups, Jacobians,
 * F evaluations, failed.  Returns the number of failed cells. */
long orc_chem_dirk_evolve(const orc_chem* c, long n, double* y, const double* scale,
                          const double* inv_scale, const double* mdens, const double* imdens,
                          const double* cie_oda, const double* h2_oda, double* Ts, double* dTs_ge,
                          const orc_dirk_opts* O, int* stats);

#ifdef __cplusplus
}
#endif
#endif
