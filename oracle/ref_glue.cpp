/* extern "C" entry points around the reference's chemistry-hydrodynamics glue, compiled
 * unmodified from the reference tree against the one-rank shims (see oracle/build_ref.sh):
 *
 *   fexpl                       src/imex_chem_hydro_main.cpp:910-1000 (a static function:
 *                               reached by including that file, its main renamed)
 *   PostprocessStep             src/imex_chem_hydro_main.cpp:1002-1051
 *   initialize / prepare / apply / unapply_Dengo_structures / _scaling
 *                               src/primordial_static.cpp:180-318
 *
 * TEST INFRASTRUCTURE ONLY: generates tests/golden/glue_cases.npz; never linked by the
 * product.  NVAR is 15 (ten species).
 */
#include <unistd.h>

#define main gbmv_ref_imex_main_unused
#include "imex_chem_hydro_main.cpp"
#undef main

// The input, output and restart routines of src/io.cpp that the main program calls: never
// reached through the callbacks wrapped here (io.cpp itself needs a full HDF5).
static void io_unreachable(const char* what) {
  fprintf(stderr, "ref_glue: %s is not available\n", what);
  abort();
}
int load_inputs(int, int, char**, EulerData&, ARKODEParameters&, int&) {
  io_unreachable("load_inputs");
  return -1;
}
int print_stats(const realtype&, N_Vector, const int&, const int&, const int&, void*,
                const EulerData&) {
  io_unreachable("print_stats");
  return -1;
}
int read_restart(const int&, realtype&, N_Vector, const EulerData&) {
  io_unreachable("read_restart");
  return -1;
}
int output_solution(const realtype&, N_Vector, const realtype&, const int&, const EulerData&,
                    const ARKODEParameters&) {
  io_unreachable("output_solution");
  return -1;
}
int check_conservation(const realtype&, N_Vector, const EulerData&) {
  io_unreachable("check_conservation");
  return -1;
}

namespace {

EulerData* g_udata = nullptr;

void as_manyvector(shim_nvector& v, double* const* fields, long n, int nchem) {
  v.nsub = 6;
  for (int k = 0; k < 6; ++k) {
    v.sub[k] = fields[k];
    v.len[k] = k < 5 ? n : n * nchem;
  }
}

}  // namespace

extern "C" {

/* EulerData for an nx x ny x nz grid on [0,1]^3 with boundary codes bc, gamma and the unit
 * scalings; the Dengo structures (rate tables from table_dir/primordial_tables.h5) prepared
 * from the physical chemistry chem_phys (10 per cell, as prepare_Dengo_structures takes it from
 * the solution vector; chem_phys is overwritten with ones, as there). */
int ref_glue_setup(long nx, long ny, long nz, const int* bc, double gamma, double mass_units,
                   double length_units, double time_units, const char* table_dir,
                   double* chem_phys) {
  delete g_udata;
  g_udata = new EulerData();
  EulerData& u = *g_udata;
  u.nx = nx; u.ny = ny; u.nz = nz;
  u.xl = 0.0; u.xr = 1.0; u.yl = 0.0; u.yr = 1.0; u.zl = 0.0; u.zr = 1.0;
  u.xlbc = bc[0]; u.xrbc = bc[1]; u.ylbc = bc[2]; u.yrbc = bc[3]; u.zlbc = bc[4]; u.zrbc = bc[5];
  u.gamma = gamma;
  u.MassUnits = mass_units;
  u.LengthUnits = length_units;
  u.TimeUnits = time_units;
  if (u.UpdateUnits() != 0) return -1;
  if (u.SetupDecomp() != 0) return -2;
  char cwd[4096];
  if (!getcwd(cwd, sizeof cwd) || chdir(table_dir) != 0) return -3;
  const int rc = initialize_Dengo_structures(u);
  if (chdir(cwd) != 0 || rc != 0) return -4;
  const long n = nx * ny * nz;
  shim_nvector w{};
  w.nsub = 6;
  for (int k = 0; k < 5; ++k) { w.sub[k] = nullptr; w.len[k] = n; }
  w.sub[5] = chem_phys;
  w.len[5] = n * u.nchem;
  realtype t = 0.0;
  return prepare_Dengo_structures(t, &w, u);
}

double ref_glue_energy_units(void) { return g_udata ? g_udata->EnergyUnits : 0.0; }

/* fexpl(t, w, wdot) of the IMEX program (w is modified as there: et, and the chemistry's
 * in-place scale / unscale round trip). */
int ref_glue_fexpl(double t, double* const* w, double* const* wdot) {
  if (!g_udata) return -100;
  const long n = g_udata->nx * g_udata->ny * g_udata->nz;
  shim_nvector a{}, b{};
  as_manyvector(a, w, n, g_udata->nchem);
  as_manyvector(b, wdot, n, g_udata->nchem);
  return fexpl(t, &a, &b, g_udata);
}

int ref_glue_postprocess(double t, double* const* w) {
  if (!g_udata) return -100;
  const long n = g_udata->nx * g_udata->ny * g_udata->nz;
  shim_nvector a{};
  as_manyvector(a, w, n, g_udata->nchem);
  return PostprocessStep(t, &a, g_udata);
}

/* apply (mode 1) or unapply (mode 0) the Dengo scaling to the chemistry of w */
int ref_glue_scaling(double* const* w, int mode) {
  if (!g_udata) return -100;
  const long n = g_udata->nx * g_udata->ny * g_udata->nz;
  shim_nvector a{};
  as_manyvector(a, w, n, g_udata->nchem);
  return mode ? apply_Dengo_scaling(&a, *g_udata) : unapply_Dengo_scaling(&a, *g_udata);
}

}  // extern "C"
