/* gbmv: GB300 (sm_103a) right-hand-side hot path of the SUNDIALS ManyVector chemistry/
 * hydrodynamics demonstration code, behind a plain C ABI.
 *
 * All array arguments are DEVICE pointers (cudaMalloc / torch CUDA storage) unless the comment
 * says "host".  `stream` is a cudaStream_t passed as void* (NULL = the legacy default stream).
 * Return codes follow the ARKODE callback convention of the reference: 0 success, >0
 * recoverable failure, <0 unrecoverable failure; the GBMV_E* codes below are all negative.
 *
 * Vector layout (the reference's MPIManyVector, one rank):
 *   component 0..4: rho, mx, my, mz, et, each nx*ny*nz doubles, x fastest
 *                   (INDX, src/euler3D.hpp:62)
 *   component 5   : chemistry/tracers, nchem*nx*ny*nz doubles, species fastest
 *                   (BUFINDX, src/euler3D.hpp:65)
 * Dense Jacobian / Newton-matrix blocks: ncells blocks of 10x10 doubles, column-major,
 *   element (row, col) of block i at [i*100 + col*10 + row] (DENSEIDX of
 *   src/raja_primordial_network.cpp:40, the SUNMatrix_MagmaDenseBlock layout).
 */
#ifndef GBMV_H
#define GBMV_H

#ifdef __cplusplus
extern "C" {
#endif

#define GBMV_OK 0
#define GBMV_ILLEGAL_STATE (-1)     /* fEuler's legal_state failure (src/utilities.cpp:83-84) */
#define GBMV_EINVAL (-101)          /* bad argument */
#define GBMV_ECUDA (-102)           /* CUDA runtime error */
#define GBMV_ENOMEM (-103)          /* device allocation failed */
#define GBMV_EUNSUPPORTED (-104)    /* NVAR / option not compiled in */

/* Boundary condition codes (src/euler3D.hpp:86-89). */
#define GBMV_BC_PERIODIC 0
#define GBMV_BC_NEUMANN 1
#define GBMV_BC_DIRICHLET 2
#define GBMV_BC_REFLECTING 3

/* Arithmetic of the WENO flux-divergence. */
#define GBMV_FP64 0   /* all arithmetic in FP64 (parity form: <=1e-12 vs the reference) */
#define GBMV_MIXED 1  /* face fluxes in float-float arithmetic on the FP32 pipes (~48-bit
                         significand, native-FP64 fallback outside the float range), divergence
                         and conservation sums in FP64 (<=1e-6 vs the FP64 oracle) */
#define GBMV_MIXED_FAST 2 /* as GBMV_MIXED, but each species (tracer) reconstruction is the
                         float-float central value plus an FP32-weighted correction built from
                         float-float neighbour differences (smoothness indicators and weights
                         in FP32 on differences, so their rounding scales with the local
                         variation, not with the value); the characteristic fluid fields keep
                         float-float weights (<=1e-6 vs the FP64 oracle) */

/* Grid + problem description: the fields of EulerData the RHS needs
 * (src/euler3D.hpp:183-253).  nchem must be one of 0, 2, 4, 6, 10 (NVAR 5, 7, 9, 11, 15,
 * the variants of src/CMakeLists.txt:29). */
typedef struct gbmv_grid {
  long nx, ny, nz;
  int nchem;
  double dx, dy, dz;
  double gamma;
  int bc[6]; /* x-lower, x-upper, y-lower, y-upper, z-lower, z-upper */
} gbmv_grid;

/* ------------------------------------------------------------------ hydro (part a) */

typedef struct gbmv_hydro_s* gbmv_hydro;

/* EulerData counterpart: validates the grid (extents >= 3, periodic faces paired, as
 * EulerData::SetupDecomp, src/euler3D.hpp:442-489) and allocates the device scratch the
 * RHS needs.  Replaces EulerData::SetupDecomp's flux-array allocation. */
int gbmv_hydro_create(const gbmv_grid* grid, gbmv_hydro* out);
int gbmv_hydro_destroy(gbmv_hydro h);

/* Constant per-field body force added to every cell (host array of NVAR doubles, NULL = 0):
 * the external_forces problem hook of the reference for constant forcings such as
 * src/rayleigh_taylor.cpp:117-128. */
int gbmv_hydro_set_force(gbmv_hydro h, const double* force_host);

/* Flags for gbmv_feuler_async. */
#define GBMV_FORCE_IN_WDOT 1 /* wdot already holds G(t) (a general external_forces); add to it */

/* fEuler (src/utilities.cpp:17-253): wdot = G - div F(w), 5th-order WENO flux divergence with
 * periodic / Neumann / Dirichlet / reflecting ghost synthesis in-kernel (replaces
 * EulerData::ExchangeStart/ExchangeEnd, src/euler3D.hpp:577-1191).  Synchronous: waits on
 * `stream` to report GBMV_ILLEGAL_STATE (-1) for a non-positive density, energy or pressure
 * anywhere (src/euler3D.hpp:1405-1414). */
int gbmv_feuler(gbmv_hydro h, double t, const double* const* w, double* const* wdot,
                int precision, void* stream);

/* Same, fully asynchronous and CUDA-graph capturable: the legal-state bit mask (1 density,
 * 2 energy, 4 pressure, OR-ed over cells) is OR-ed into *d_status (device int). */
int gbmv_feuler_async(gbmv_hydro h, double t, const double* const* w, double* const* wdot,
                      int precision, int flags, int* d_status, void* stream);

/* fEuler without any device allocation.  This entry point has no counterpart in the
 * reference; it exists for callers that cannot call cudaMalloc: code running under a
 * fixed device-memory budget handed out by someone else (an integrator or application
 * that owns every byte of HBM through its own pool), or code paths where allocating would
 * synchronise the device at a moment the caller cannot afford.  It computes exactly what
 * gbmv_feuler computes in the FP64 form (no handle needed: grid and the NVAR per-field force
 * constants, host array or NULL, are passed directly), using a face-flux scratch array and a
 * status word that are fixed-size __device__ arrays inside this library instead of
 * cudaMalloc'ed buffers.
 *   Limit: (5+nchem) * [(nx+1)*ny*nz + nx*(ny+1)*nz + nx*ny*(nz+1)] <= 8388608 doubles
 *          (64 MiB, e.g. 56^3 at nchem=10, 82^3 at nchem=0); larger grids return GBMV_EINVAL
 *          with a message, nothing is launched.  Bad grids, null fields: the codes and
 *          messages of gbmv_hydro_create / gbmv_feuler.
 *   The first call on each device looks up the arrays' device addresses (with that device
 *   current).  Under CUDA's lazy module loading (the default) that lookup is also what commits
 *   the 64 MiB on the device, which then stays committed until the process exits.  So make
 *   the first call on each device before the caller's memory pool takes the device's free
 *   memory, and before any stream capture; later calls commit nothing more.
 *   All calls share the one array and status word, which keep the last call's contents: the
 *   status word is cleared at the start of each call, but calls that overlap on the GPU
 *   (other streams, other host threads) race on the shared scratch -- serialise them.
 *   Synchronous on `stream` like gbmv_feuler; returns 0, GBMV_ILLEGAL_STATE, or < 0. */
int gbmv_feuler_noalloc(const gbmv_grid* grid, const double* force_host, double t,
                        const double* const* w, double* const* wdot, void* stream);

/* Autotuner of the face sweeps' launch shape (no counterpart in the reference): times the
 * flux divergence of `precision` on the state w with 32, 64 and 128 threads per block and
 * keeps the fastest for this handle and precision (*threads, host, may be NULL, receives it).
 * Each face is computed by one thread on its own, so the choice changes no result.  Without a
 * call the sweeps use 128 threads, fewer on grids too small to give every SM two blocks.
 * Synchronous; allocates a temporary output; not during a stream capture. */
int gbmv_hydro_autotune(gbmv_hydro h, const double* const* w, int precision, int* threads,
                        void* stream);

/* Register budget of the GBMV_MIXED_FAST face sweeps (no counterpart in the reference):
 * GBMV_SWEEPS_ALONE (default) sizes them to run alone on the GPU (3 resident 128-thread blocks
 * per SM); GBMV_SWEEPS_SHARED for running beside another kernel on the same SMs, e.g. the
 * chemistry Newton on a second stream of the same CUDA graph (5 blocks per SM: fewer registers
 * a thread, so the other kernel's warps fit beside them).  The sweeps compute the same values
 * bit for bit under either budget; only the speed differs.  Takes effect at the next launch
 * (a captured graph keeps the budget it was captured with). */
#define GBMV_SWEEPS_ALONE 0
#define GBMV_SWEEPS_SHARED 1
int gbmv_hydro_set_sweep_budget(gbmv_hydro h, int budget);

/* Threads per block of the face sweeps of `precision` on this handle: 32, 64 or 128, or 0 for
 * the size-based default -- what gbmv_hydro_autotune picks, set by a caller that tunes a
 * composition of its own (for example the sweeps beside the chemistry Newton).  Results do not
 * depend on it.  Returns 0 or GBMV_EINVAL. */
int gbmv_hydro_set_sweep_threads(gbmv_hydro h, int precision, int threads);

/* stability (src/utilities.cpp:483-528): dt_stab = cfl * min(dx,dy,dz) / max(|mx/rho| + c),
 * including the reference's use of |mx/rho| for all three directions.  *dt_stab is host. */
int gbmv_stability(gbmv_hydro h, const double* const* w, double cfl, double* dt_stab,
                   void* stream);

/* Derivatives of fEuler in its FP64 form (no counterpart in the reference, which has no
 * adjoint; for Newton-Krylov Jacobian actions, sensitivities and gradients through time steps):
 *   gbmv_feuler_jvp: jv = (d fEuler / d w)(w) dw  (forward mode: the face flux on dual
 *                    numbers, the exact linearisation of what gbmv_feuler computes);
 *   gbmv_feuler_vjp: u = (d fEuler / d w)(w)^T v  (hand-written reverse mode of the face flux
 *                    and the divergence, ghost rules inverted; deterministic, no atomics).
 * All arguments are ManyVectors laid out like w.  The constant external force has no
 * derivative.  At kinks (the Lax-Friedrichs max over the stencil, |u|) the branch the forward
 * evaluation took is differentiated.  The first VJP call on a handle allocates
 * 6 (5+nchem) x (faces of one direction) doubles: make it before any stream capture.
 * Asynchronous; returns 0 or < 0. */
int gbmv_feuler_jvp(gbmv_hydro h, double t, const double* const* w, const double* const* dw,
                    double* const* jv, void* stream);
int gbmv_feuler_vjp(gbmv_hydro h, double t, const double* const* w, const double* const* v,
                    double* const* u, void* stream);

/* Cells where a central difference of fEuler along dw crosses a kink (no counterpart in the
 * reference; for derivative tests): mask[cell] = 1 (device, ncells bytes) when one of the
 * cell's six faces changes its Lax-Friedrichs branch -- the stencil point that maximises
 * |u| + c, or the sign of that point's velocity -- between w - eps dw, w and w + eps dw;
 * elsewhere (f(w + eps dw) - f(w - eps dw)) / (2 eps) differentiates one smooth branch and
 * converges to gbmv_feuler_jvp.  Asynchronous. */
int gbmv_feuler_kink_mask(gbmv_hydro h, const double* const* w, const double* const* dw,
                          double eps, unsigned char* mask, void* stream);

/* pack1D_x / pack1D_y / pack1D_z and their _bdry variants (EulerData, src/euler3D.hpp:
 * 1197-1378), for all faces at once: the six-point stencils the face fluxes of direction dir
 * (0 x, 1 y, 2 z) read, after the periodic wrap and the boundary ghost rules.  out (device):
 * 6 * (5+nchem) * nfaces doubles, out[(l * (5+nchem) + v) * nfaces + f], f the face index
 * i + (nx+1) (j + ny k) for x faces (y, z likewise), stencil point l = 0..5 at cell index
 * (face - 3 + l) along dir, v in ManyVector field order.  Asynchronous. */
int gbmv_pack1d(gbmv_hydro h, const double* const* w, int dir, double* out, void* stream);

/* check_conservation (src/io.cpp:503-542): totals[0] = mass_factor * sum(rho),
 * totals[1] = energy_factor * sum(et) over all cells, with the reference's factors
 * mass_factor = dx dy dz LengthUnits^3 DensityUnits, energy_factor = dx dy dz LengthUnits^3
 * EnergyUnits (pass 1, 1 for the raw sums).  FP64, compensated and deterministic (fixed
 * reduction order, no atomics).  totals is host memory; synchronous. */
int gbmv_conservation(gbmv_hydro h, const double* const* w, double mass_factor,
                      double energy_factor, double* totals, void* stream);

/* N_VWrmsNorm of a ManyVector with ARKODE's error weights (the norm ARKStep's error test and
 * its Newton convergence test take after ARKStepSVtolerances, src/imex_chem_hydro_main.cpp:463,
 * and the MRIStep / ERKStep equivalents): *norm = sqrt(sum (v_i ewt_i)^2 / N), ewt_i =
 * 1 / (rtol |y_i| + atol), over the five fluid fields and the chemistry field of the handle's
 * grid (N = (5 + nchem) ncells).  FP64, compensated and deterministic.  norm is host memory;
 * synchronous.  Returns 0, or GBMV_EINVAL for null pointers or rtol, atol < 0 (or both 0). */
int gbmv_wrms_norm(gbmv_hydro h, const double* const* v, const double* const* y, double rtol,
                   double atol, double* norm, void* stream);

/* print_stats (src/io.cpp:552-640): rms[v] = sqrt(sum over cells of (w_v * units_v)^2 / ncells)
 * for the 5 + nchem fields, units_v = density_units for rho, momentum_units for mx, my, mz,
 * energy_units for et (all 1 for the dimensionless output, the reference's units = 0), the
 * chemistry fields as stored.  FP64, compensated and deterministic.  rms is host memory (5 +
 * nchem doubles); synchronous. */
int gbmv_print_stats(gbmv_hydro h, const double* const* w, double density_units,
                     double momentum_units, double energy_units, double* rms, void* stream);

/* -------------------------------------------------------------- chemistry (part b) */

typedef struct gbmv_chem_s* gbmv_chem;

/* cvklu_data counterpart (cvklu_setup_data, src/raja_primordial_network.cpp:45-254):
 * `tables_host` is the (50 x 1024) table block in the order rates k01..k22 (no k20),
 * 25 cooling terms, 4 H2 adiabatic-index tables (see h5tables.TABLE_NAMES); Ts starts at
 * 1000 K; scale and inv_scale start at 1. */
int gbmv_chem_create(long ncells, const double* tables_host, double current_z,
                     gbmv_chem* out);
int gbmv_chem_destroy(gbmv_chem c);

/* prepare_Dengo_structures (src/primordial_static.cpp:227-259): scale = chem,
 * inv_scale = 1/chem, chem = 1, then setting_up_extra_variables
 * (src/raja_primordial_network.cpp:1969-2018). */
int gbmv_chem_prepare(gbmv_chem c, double* chem, void* stream);

/* Sets scale (device, 10*ncells) directly, inv_scale = 1/scale, and the auxiliary arrays. */
int gbmv_chem_set_scale(gbmv_chem c, const double* scale, void* stream);

/* apply_Dengo_scaling / unapply_Dengo_scaling (src/primordial_static.cpp:264-318). */
int gbmv_chem_apply_scaling(gbmv_chem c, double* chem, void* stream);
int gbmv_chem_unapply_scaling(gbmv_chem c, double* chem, void* stream);

/* calculate_rhs_cvklu (src/raja_primordial_network.cpp:1015-1389) followed by the
 * N_VScale(TimeUnits) of ffast/fimpl (src/multirate_chem_hydro_main.cpp:918-920):
 * ydot = time_units * f(y).  Updates the per-cell temperature state (Ts, dTs/dge) that the
 * next call and the Jacobian use. */
int gbmv_chem_rhs(gbmv_chem c, double t, const double* y, double* ydot, double time_units,
                  void* stream);

/* calculate_jacobian_cvklu (src/raja_primordial_network.cpp:1393-1965) in dense blocks,
 * times time_units (Jfast/Jimpl, src/multirate_chem_hydro_main.cpp:976-983). */
int gbmv_chem_jac(gbmv_chem c, double t, const double* y, double* J, double time_units,
                  void* stream);

/* One batched Newton iteration of the implicit chemistry stage, fused (no Jacobian in HBM):
 *   f = time_units * f_chem(y)           -- exactly gbmv_chem_rhs (temperature state updated)
 *   x = (I - gamma * J(y))^{-1} f        -- J as gbmv_chem_jac, A as gbmv_block_form_newton,
 *                                           solve as gbmv_block_lu_factor + _solve
 * i.e. Jfast/Jimpl + ARKLS setup + Solve_RankLocalLS of src/multirate_chem_hydro_main.cpp:
 * 954-1395 for one right-hand side, in one kernel.  lu_precision: GBMV_FP64 (FP64 LU) or
 * GBMV_MIXED (FP32 LU + `refine` iterative-refinement steps against FP64 residuals, FP64
 * fallback for blocks whose FP32 factor fails).  Returns 0, or 1 if a block is singular. */
int gbmv_chem_newton(gbmv_chem c, double t, const double* y, double* f, double* x,
                     double gamma, double time_units, int lu_precision, int refine,
                     void* stream);

/* Implicit-stage form of gbmv_chem_newton: f = TimeUnits * f(y) and
 *   x = (I - gamma * J(y))^{-1} (b + gamma * f)
 * -- one full Newton correction of the stage equation z = a + gamma f(z) at the iterate y = z
 * with b = a - z, the Newton matrix formed afresh at y (the ARKStep implicit stage of
 * src/imex_chem_hydro_main.cpp with fimpl, Jimpl and the block solver fused per cell).  Same
 * precisions and return values as gbmv_chem_newton; b, f, x: 10 * ncells doubles. */
int gbmv_chem_newton_stage(gbmv_chem c, double t, const double* y, const double* b, double* f,
                           double* x, double gamma, double time_units, int lu_precision,
                           int refine, void* stream);

/* Same, asynchronous and CUDA-graph capturable: a singular block raises *d_info (device int,
 * atomicMax to 1) instead of being returned. */
int gbmv_chem_newton_async(gbmv_chem c, double t, const double* y, double* f, double* x,
                           double gamma, double time_units, int lu_precision, int refine,
                           int* d_info, void* stream);

/* Work-queue form of gbmv_chem_newton_async (no counterpart in the reference): the launch's
 * one-warp blocks take 32-cell chunks from the device counter *d_queue until every cell is
 * taken, so several launches -- on different streams of one graph -- can share one pass over
 * the cells: for example a narrow persistent launch beside the WENO sweep of the stage and a
 * wide one after the sweep that drains what is left.  The caller zeroes *d_queue before the
 * first launch that shares it.  blocks_per_sm: 0 = a deep grid (as many blocks as fit), n > 0
 * = n resident one-warp blocks per SM.  Every cell's f and x are those of
 * gbmv_chem_newton_async bit for bit, whichever launch computes it. */
int gbmv_chem_newton_queue_async(gbmv_chem c, double t, const double* y, double* f, double* x,
                                 double gamma, double time_units, int lu_precision, int refine,
                                 unsigned long long* d_queue, int blocks_per_sm, int* d_info,
                                 void* stream);

/* Products with the chemistry Jacobian of gbmv_chem_jac (J = time_units * df/dy at the
 * temperature state of the last gbmv_chem_rhs, entries rounded exactly as gbmv_chem_jac
 * writes them) without forming it: gbmv_chem_jvp jv = J dy (the matrix-free Jacobian action
 * of Newton-Krylov), gbmv_chem_vjp u = J^T v (the adjoint of the chemistry source).
 * 10 * ncells doubles each.  Asynchronous. */
int gbmv_chem_jvp(gbmv_chem c, double t, const double* y, const double* dy, double* jv,
                  double time_units, void* stream);
int gbmv_chem_vjp(gbmv_chem c, double t, const double* y, const double* v, double* u,
                  double time_units, void* stream);

/* Options of the persistent DIRK chemistry integrator (gbmv_chem_dirk_evolve). */
typedef struct {
  double rtol, atol; /* WRMS weights 1 / (rtol |z| + atol) on the scaled variables */
  double nlscoef;    /* Newton convergence factor (ARKODE's nlscoef; default 0.1) */
  double h0;         /* first step in time units of t; <= 0: from ||F(z0)|| (default 0) */
  double safety;     /* step-size safety factor (default 0.9) */
  double dgmax;      /* refactor when |gamma / gamma_p - 1| > dgmax (default 0.2) */
  double growth;     /* largest step growth after the first step (default 20) */
  double etamx1;     /* largest growth on the first step (default 10000) */
  double hmax;       /* largest step, <= 0: none (default 0) */
  int maxcor;        /* Newton iterations per stage (default 3) */
  int max_steps;     /* steps per cell before it counts as failed (default 5000) */
  int msbp;          /* new Newton matrix (fresh J, refactored) at least every msbp steps
                        (default 20) */
  int maxnef;        /* error-test failures per step (default 7) */
  int maxncf;        /* Newton failures per step (default 10) */
  int precision;     /* GBMV_FP64: FP64 LU and temperature; GBMV_MIXED: FP32 LU (+ refine),
                        temperature iterations 1-8 in FP32 (default GBMV_FP64) */
  int refine;        /* GBMV_MIXED: FP64-residual refinement steps per linear solve, 0-8;
                        > 0 keeps an FP64 copy of the matrix (default 0: each Newton
                        iteration already refines against the FP64 nonlinear residual) */
  int block;         /* threads per block: 32, 64 or 128; 0 = autotuned (default 0) */
  int table;         /* ARKODE DIRK table number (the `itable` input option): 112
                        ARK437L2SA_DIRK_7_3_4 (the reference's chemistry inputs, default) or 102
                        TRBDF2_3_3_2; any stiffly accurate ESDIRK of gbmv_butcher_table with an
                        explicit first stage and one diagonal value is accepted */
  int setup_batch;   /* Newton-matrix setups are gathered per warp: a cell that needs one waits
                        (no F evaluation) until this many cells of its warp wait, or every
                        active cell of the warp waits, or one has waited 4 x setup_batch
                        passes, or no cell is left to start; then they set up together.  1 =
                        every cell sets up at once.  Every cell runs the same computation
                        whatever the value: only the interleaving changes (default 8) */
  int order;         /* 1: cells are taken largest initial derivative first (||F(z0)|| in the
                        WRMS norm, in quarter-decade buckets), so the costliest cells start
                        early and few lanes idle at the end; 0: in index order.  Every cell's
                        result is the same either way (default 1) */
  int deduce;        /* 1: the derivative of every converged intermediate stage is deduced
                        from its stage equation, K_i = (z_i - base_i) / (h gamma), instead of
                        evaluating F(z_i) (ARKODE's ARKStepSetDeduceImplicitRhs; a Newton error
                        enters K_i as itself over h gamma rather than multiplied by the stiff
                        Jacobian); the last stage is still evaluated, since F(z_s) = F(y_{n+1})
                        is the next step's first stage.  In the GBMV_MIXED form the FP32 pass
                        also hands a cell to the FP64-factor pass after 8 Newton failures in
                        all (a deduced derivative carries the FP32 factor's inexact
                        corrections).  0: every stage evaluated, ARKODE's default (default 0) */
} gbmv_dirk_opts;

/* Fill *o with the defaults above (rtol 1e-6, atol 1e-10). */
void gbmv_dirk_opts_default(gbmv_dirk_opts* o);

/* Integrate every cell's chemistry dz/dt = time_units * f_chem(z) (scaled variables, as
 * gbmv_chem_rhs) from t0 to tout with the adaptive ESDIRK of opts->table and modified Newton
 * on per-cell 10x10 systems, each cell on its own step sequence, in one persistent launch
 * that retires finished cells and pulls new ones.  In the GBMV_MIXED form the cells whose
 * FP32 pass fails are integrated again from their start state by a second launch with the
 * FP64 factor over just those cells (counted by gbmv_chem_dirk_retried).  It replaces the fast-stage
 * integration of the chemistry drivers: ARKStep DIRK + Jfast/Jimpl + the block solver
 * (src/primordial_ode_main.cpp) and the rank-local MRI inner stepper's evolve
 * (src/multirate_chem_hydro_main.cpp:1114-1224), with per-cell instead of rank-wide step
 * control.  y: 10 * ncells device doubles, updated in place; the temperature state is
 * carried.  stats: NULL or 8 device ints per cell (steps, Newton iterations, error-test
 * failures, Newton failures, matrix setups, Jacobian evaluations, F evaluations, failed).
 * With opts->block == 0 the first call per precision times each block size on a sample of
 * the cells (state restored) and keeps the fastest: make that call before any stream capture.
 * Returns the number of failed cells (>= 0; their y holds the last accepted step) or a
 * negative GBMV_E* code.  Synchronous. */
int gbmv_chem_dirk_evolve(gbmv_chem c, double t0, double tout, double* y, double time_units,
                          const gbmv_dirk_opts* opts, int* stats, void* stream);

/* Same, asynchronous and graph-capturable (opts->block must be set, or tuned by an earlier
 * call): the failed-cell count is added to *d_nfail (device int, caller-zeroed). */
int gbmv_chem_dirk_evolve_async(gbmv_chem c, double t0, double tout, double* y,
                                double time_units, const gbmv_dirk_opts* opts, int* stats,
                                int* d_nfail, void* stream);

/* The rank-local MRI inner stepper's evolve (RankLocalStepper_Evolve,
 * src/multirate_chem_hydro_main.cpp:1114-1160: ARKStepEvolve of ffast to tout) on the GPU:
 * advances the fast problem w' = ffast(t, w) (see gbmv_ffast) from t0 to tout.  The
 * chemistry component w[5] is integrated by the persistent DIRK of gbmv_chem_dirk_evolve with
 * the forcing's chemistry component added to its right-hand side at every stage time; the
 * fluid components, whose fast tendency is the forcing polynomial alone, receive its exact
 * integral, w[k] += sum_i forcing[i*6+k] * tscale * (tau_out^(i+1) - tau_0^(i+1)) / (i+1).
 * forcing/tshift/tscale as gbmv_ffast (MRIStepInnerStepper_GetForcingData).  Returns the
 * number of failed cells (>= 0) or a negative code.  Synchronous. */
int gbmv_mri_fast_evolve(gbmv_hydro h, gbmv_chem c, double t0, double tout, double* const* w,
                         double time_units, int nforcing, const double* const* forcing,
                         double tshift, double tscale, const gbmv_dirk_opts* opts, int* stats,
                         void* stream);

/* Same, asynchronous and CUDA-graph capturable (the stage of a captured MRI slow step): the
 * failed-cell count is added to *d_nfail (device int, caller-zeroed); opts->block must be set
 * or tuned by an earlier synchronous call, and the first call on the handle (which allocates
 * the DIRK stage store) must come before any capture. */
int gbmv_mri_fast_evolve_async(gbmv_hydro h, gbmv_chem c, double t0, double tout,
                               double* const* w, double time_units, int nforcing,
                               const double* const* forcing, double tshift, double tscale,
                               const gbmv_dirk_opts* opts, int* stats, int* d_nfail,
                               void* stream);

/* The GBMV_MIXED DIRK (refine 0) runs two passes: every cell in FP32-LU arithmetic, then the
 * cells that pass could not finish (Newton iterations that keep failing on an FP32 factor too
 * poor for the block) again from their start state with the FP64 factor (and the mixed
 * temperature solve, within ~1e-16 of the FP64 form's), so they end where the FP64 form ends
 * them to rounding.  This returns how many cells the last GBMV_MIXED call on the handle sent to
 * the second pass, and copies up to max_cells of their indices (host) into cells (may be NULL).
 * Synchronous. */
int gbmv_chem_dirk_retried(gbmv_chem c, int* cells, int max_cells, void* stream);

/* Block size the autotuner chose for a precision (0 = not tuned yet). */
int gbmv_chem_dirk_block(gbmv_chem c, int precision);

/* Launch shape of gbmv_chem_newton(_async) on this handle: 0 (default) a deep grid-stride
 * grid; n > 0 exactly n resident 64-thread blocks per SM, a persistent grid that leaves room
 * on every SM for a kernel running beside it on another stream (for example the WENO sweep of
 * the same stage: the chemistry and the flux divergence of a stage are independent and load
 * different pipes, FP64 and FP32).  Returns 0 or GBMV_EINVAL. */
int gbmv_chem_set_newton_occupancy(gbmv_chem c, int blocks_per_sm);

/* Autotuner of gbmv_chem_newton's launch shape: times the fused Newton on y (gamma,
 * time_units, lu_precision, refine as the caller will use them) on the deep grid-stride grid
 * and on persistent grids of 2-8 one-warp blocks per SM, restores the temperature state, and
 * keeps the fastest as the handle's Newton occupancy (as gbmv_chem_set_newton_occupancy;
 * *blocks_per_sm, host, may be NULL, receives it, 0 = the deep grid).  Per-cell work does not
 * depend on the launch shape, so results are unchanged.  Synchronous; not during a capture. */
int gbmv_chem_newton_autotune(gbmv_chem c, const double* y, double gamma, double time_units,
                              int lu_precision, int refine, int* blocks_per_sm, void* stream);

/* Device pointers of the persistent per-cell state (for checkpoint/restart and tests):
 * which: 0 Ts, 1 dTs_ge, 2 mdensity, 3 inv_mdensity, 4 cie optical depth, 5 h2 optical depth,
 * 6 scale, 7 inv_scale. */
double* gbmv_chem_state(gbmv_chem c, int which);

/* ---------------------------------------------------- block-diagonal solve (part c) */

/* SUNLinSolSetup of the MAGMA batched dense solver wrapped by SUNLinSol_RankLocalLS /
 * SUNLinSol_BDMPIMV (src/multirate_chem_hydro_main.cpp:1360-1369,
 * src/imex_chem_hydro_main.cpp:1123-1132): LU with partial pivoting of every 10x10 block of
 * A in place; pivots: 10 ints per block.  Returns 0, or a positive value (SUNLS_LUFACT_FAIL
 * style, recoverable) if some block is singular.  Synchronous.  The singular-block flag is a
 * device word of the calling host thread on the current device (allocated at that thread's
 * first call there), so calls from different threads or on different devices do not share
 * it. */
int gbmv_block_lu_factor(long nblocks, double* A, int* pivots, void* stream);

/* SUNLinSolSolve of the same (src/multirate_chem_hydro_main.cpp:1371-1395): x = A^{-1} b
 * on the chemistry subvector; b and x may alias. */
int gbmv_block_lu_solve(long nblocks, const double* LU, const int* pivots, const double* b,
                        double* x, void* stream);

/* The same solver as a handle that owns its pivots (10 ints per block) and its own
 * singular-block word, the content a SUNLinearSolver built over these calls keeps
 * (SUNLinSol_RankLocalLS / SUNLinSol_BDMPIMV's block solver, src/multirate_chem_hydro_main.cpp:
 * 1312-1411).  setup factors A in place (synchronous, returns 0 or 1 for a singular block);
 * solve is asynchronous. */
typedef struct gbmv_block_ls_s* gbmv_block_ls;
int gbmv_block_ls_create(long nblocks, gbmv_block_ls* out);
int gbmv_block_ls_destroy(gbmv_block_ls ls);
int gbmv_block_ls_setup(gbmv_block_ls ls, double* A, void* stream);
int gbmv_block_ls_solve(gbmv_block_ls ls, const double* LU, const double* b, double* x,
                        void* stream);

/* ARKLS's Newton matrix A = I - gamma*J (SUNMatScaleAddI) for dense blocks, in place. */
int gbmv_block_form_newton(long nblocks, double* J, double gamma, void* stream);

/* ------------------------------------------------------ chemistry-hydro glue */

/* fslow / fexpl (src/multirate_chem_hydro_main.cpp:996-1083, src/imex_chem_hydro_main.cpp:
 * 910-1000): apply the Dengo scaling to w[5], set et = ge/EnergyUnits + |m|^2/(2 rho) in w[4],
 * evaluate fEuler, move the total-energy tendency into the gas-energy species of wdot[5]
 * (etdot = 0), undo the scaling.  GBMV_FP64 reproduces the reference's in-place scale and
 * unscale of w[5] (and its rounding); GBMV_MIXED leaves w[5] untouched (the scale is applied
 * where the WENO reads the species), so w[5] may be read concurrently, e.g. by the chemistry
 * of the same stage on another stream.  Synchronous like gbmv_feuler. */
int gbmv_fexpl(gbmv_hydro h, gbmv_chem c, double t, double* const* w, double* const* wdot,
               double energy_units, int precision, void* stream);

/* ffast (src/multirate_chem_hydro_main.cpp:897-946), the fast right-hand side of the
 * multirate driver: wdot[0..4] = 0, wdot[5] = time_units * f_chem(w[5]) (as gbmv_chem_rhs),
 * then the MRI inner-stepper forcing on all six components,
 *   wdot[k] += sum_{i < nforcing} tau^i forcing[i*6 + k],   tau = (t - tshift) / tscale,
 * (MRIStepInnerStepper_GetForcingData + N_VLinearCombination).  forcing: host array of
 * nforcing*6 device pointers laid out like w (NULL when nforcing == 0); nforcing <= 8.
 * Asynchronous (no status to report). */
int gbmv_ffast(gbmv_hydro h, gbmv_chem c, double t, const double* const* w, double* const* wdot,
               double time_units, int nforcing, const double* const* forcing, double tshift,
               double tscale, void* stream);

/* Same, asynchronous and CUDA-graph capturable: the legal-state mask is OR-ed into
 * *d_status (device int) instead of being returned. */
int gbmv_fexpl_async(gbmv_hydro h, gbmv_chem c, double t, double* const* w,
                     double* const* wdot, double energy_units, int precision, int* d_status,
                     void* stream);

/* PostprocessStep (src/imex_chem_hydro_main.cpp:1002-1051): et from ge and momenta. */
int gbmv_postprocess_step(gbmv_hydro h, gbmv_chem c, double* const* w, double energy_units,
                          void* stream);

/* ------------------------------------------------------------ Butcher tables */

/* The Runge-Kutta tables the reference's input files select, by ARKODE table number (the
 * `etable` / `itable` options of src/euler3D.hpp:126-172, given to ARKStepSetTableNum in
 * src/euler3D_main.cpp:209-213, src/imex_chem_hydro_main.cpp:386 and
 * src/multirate_chem_hydro_main.cpp:447), with the published coefficients:
 *   explicit: 0 HEUN_EULER_2_1_2, 1 BOGACKI_SHAMPINE_4_2_3, 2 ARK324L2SA_ERK_4_2_3,
 *             3 ZONNEVELD_5_3_4, 6 CASH_KARP_6_4_5, 8 DORMAND_PRINCE_7_4_5,
 *             13 ARK437L2SA_ERK_7_3_4;
 *   implicit: 102 TRBDF2_3_3_2, 104 ARK324L2SA_DIRK_4_2_3, 112 ARK437L2SA_DIRK_7_3_4.
 * (2, 104) and (13, 112) are additive IMEX pairs (shared c and b).  Host-only: no device work. */
#define GBMV_MAX_STAGES 7
typedef struct {
  int id;
  int stages;   /* s */
  int q;        /* method order */
  int p;        /* embedding order */
  double c[GBMV_MAX_STAGES];
  double A[GBMV_MAX_STAGES][GBMV_MAX_STAGES]; /* row-major, diagonal included */
  double b[GBMV_MAX_STAGES];
  double bhat[GBMV_MAX_STAGES];
  char name[32];
} gbmv_butcher;

/* Fill *out with table `id`; returns 0 or GBMV_EUNSUPPORTED (with a message). */
int gbmv_butcher_table(int id, gbmv_butcher* out);

/* ARKODE's default explicit table for an `order` (ARKStepSetOrder, the `order` input option,
 * src/euler3D_main.cpp:207-209): 2 -> 0, 3 -> 1, 4 -> 3, 5 -> 6; -1 for other orders. */
int gbmv_erk_default_table(int order);

/* ------------------------------------------------ device-resident step control */

/* Adaptive time stepping whose every step is a CUDA graph (the stages, the error norm and
 * these calls captured once and replayed): the accept / reject decision and the step-size
 * controller run on the device, so the host reads nothing back between steps.  No
 * counterpart in the reference, whose ARKStep decides on the host after a synchronising norm;
 * the controller is ARKODE's (ARKStepSetAdaptivityMethod's PID / PI / I with k1, k2, k3,
 * safety, bias, growth, etamx1, etamxf, small_nef; src/euler3D.hpp:126-172 options).
 * The state is GBMV_STEP_STATE doubles of device memory at the indices below; initialise it
 * with t = t0, tf, h = the first step, first = 1, e1 = e2 = 1, everything else 0 (a graph
 * captured over these calls serves any interval: the interval lives in the state). */
#define GBMV_ST_T 0        /* current time */
#define GBMV_ST_H 1        /* proposed next step */
#define GBMV_ST_HUSED 2    /* the step of the attempt in flight (0 when done) */
#define GBMV_ST_ACCEPT 3   /* 1 if the last attempt was accepted */
#define GBMV_ST_DONE 4     /* 1 once t reached tf or the run failed */
#define GBMV_ST_E1 5       /* bias * dsm of the last accepted step */
#define GBMV_ST_E2 6       /* ... and of the one before */
#define GBMV_ST_FIRST 7    /* 1 before the first accepted step */
#define GBMV_ST_NEF 8      /* error-test failures of the step in progress */
#define GBMV_ST_STEPS 9    /* accepted steps */
#define GBMV_ST_ATTEMPTS 10
#define GBMV_ST_FAILS 11   /* error-test failures */
#define GBMV_ST_STATUS 12  /* 0, -1 maxnef failures in one step, -2 max_attempts reached */
#define GBMV_ST_LAST 13    /* 1 if the attempt in flight ends on tf */
#define GBMV_ST_HPROP 14   /* the proposal before the cut to tf */
#define GBMV_ST_TF 15      /* end of the integration interval */
#define GBMV_STEP_STATE 16

typedef struct {
  double hmax;           /* largest step (0: none) */
  double safety, bias, growth, etamx1, etamxf;
  double k1, k2, k3;     /* controller gains (k2 = k3 = 0: I controller; k3 = 0: PI) */
  int order;             /* the order k in the exponents (the embedding order) */
  int small_nef, maxnef, max_attempts;
  int fixed;             /* 1: fixed steps of h, no error control */
} gbmv_step_params;

/* Start an attempt: h_used = min(h, hmax, tf - t) (0 and done = 1 when nothing is left). */
int gbmv_step_begin(double* d_state, const gbmv_step_params* p, void* stream);
/* Finish it with the WRMS error norm *d_dsm (device): accept (t += h_used) or reject, next h
 * from the controller; failures set status and done. */
int gbmv_step_end(double* d_state, const double* d_dsm, const gbmv_step_params* p, void* stream);
/* y = ynew over n doubles if the last attempt was accepted (else nothing). */
int gbmv_step_select(long n, const double* d_state, double* y, const double* ynew, void* stream);

/* gbmv_wrms_norm with the result in device memory (*d_norm) and no synchronisation, for
 * step graphs; the handle's reduction scratch must exist already (any earlier synchronous
 * reduction call on the handle, or one call of this outside a capture). */
int gbmv_wrms_norm_async(gbmv_hydro h, const double* const* v, const double* const* y,
                         double rtol, double atol, double* d_norm, void* stream);

/* ----------------------------------------------------------------- utilities */

const char* gbmv_version(void);
const char* gbmv_last_error(void);
/* Number of kernel launches issued by this library since load (for launch accounting). */
long gbmv_launch_count(void);

/* Per-kernel-family timing with CUDA events recorded on the launching stream (no counterpart
 * in the reference, which times with MPI_Wtime in src/profiler.hpp).  Families:
 * "face_flux", "divergence", "chem_rhs", "chem_jac", "block_lu_factor", "block_lu_solve",
 * "glue".  gbmv_profile_get synchronizes on the recorded events. */
int gbmv_profile_enable(int on);
int gbmv_profile_reset(void);
int gbmv_profile_get(const char* family, double* total_ms, long* launches);

/* Diagnostics (no counterpart in the reference): peak FMA throughput of the SIMT pipes,
 * FP64 (fp64=1) or FP32 (fp64=0), in flop/s (2 per FMA) -- the FP64 roofline denominator. */
int gbmv_diag_fma_rate(int fp64, double* flops_per_s);

/* Self-check of the integer-instruction double <-> float conversions the mixed kernels use in
 * place of conversion instructions (which run at the FP64 rate): for each of the n device
 * doubles, the conversions and float-pair splits must match the hardware round-to-nearest
 * results bit for bit; *mismatches (host) counts the differences.  Synchronous.  (No
 * counterpart in the reference.) */
int gbmv_diag_convert_check(const double* d_in, long n, unsigned long long* mismatches,
                            void* stream);

#ifdef __cplusplus
}
#endif
#endif
