/* extern "C" entry points around the reference's own hot-path code, compiled unmodified
 * from the reference tree against oracle/ref_shim (see oracle/build_ref.sh).
 *
 * TEST INFRASTRUCTURE ONLY.  Used to (1) validate the oracle restatement in oracle/oracle.c
 * and (2) generate the golden fixtures under tests/golden/.  Never linked by the product.
 *
 * Wraps:
 *   fEuler                      src/utilities.cpp:17-253   (with face_flux :270-479)
 *   EulerData::SetupDecomp      src/euler3D.hpp:396-574    (one rank)
 *   cvklu_setup_data            src/raja_primordial_network.cpp:45-254
 *   setting_up_extra_variables  src/raja_primordial_network.cpp:1969-2018
 *   calculate_rhs_cvklu         src/raja_primordial_network.cpp:1015-1389
 *   calculate_jacobian_cvklu    src/raja_primordial_network.cpp:1393-1965 (CSR branch)
 */
#include <euler3D.hpp>
#include <raja_primordial_network.hpp>

#include <vector>

// Problem hook that every reference problem file defines (e.g. src/rayleigh_taylor.cpp:117-128):
// here a constant per-field body force, zero by default.
static double g_force[NVAR];

int external_forces(const realtype& t, N_Vector G, const EulerData& udata) {
  (void)t;
  const long n = udata.nxl * udata.nyl * udata.nzl;
  for (int v = 0; v < 5; ++v) {
    double* g = N_VGetSubvectorArrayPointer_MPIManyVector(G, v);
    for (long i = 0; i < n; ++i) g[i] = g_force[v];
  }
  if (udata.nchem > 0) {
    double* g = N_VGetSubvectorArrayPointer_MPIManyVector(G, 5);
    for (long i = 0; i < n; ++i)
      for (int c = 0; c < udata.nchem; ++c) g[c + udata.nchem * i] = g_force[5 + c];
  }
  return 0;
}

extern "C" {

int ref_nvar(void) { return NVAR; }

/* One fEuler evaluation.  fields/out: 5 SoA fluid arrays (n each) then the AoS chemistry array
 * (nchem*n) when NVAR>5.  bc: xl,xr,yl,yr,zl,zr boundary types.  force: NVAR constants. */
int ref_feuler(long nx, long ny, long nz, const double* dom, const int* bc, double gamma,
               double t, const double* force, double* const* fields, double* const* out,
               double* seconds) {
  EulerData udata;
  udata.nx = nx; udata.ny = ny; udata.nz = nz;
  udata.xl = dom[0]; udata.xr = dom[1]; udata.yl = dom[2]; udata.yr = dom[3];
  udata.zl = dom[4]; udata.zr = dom[5];
  udata.xlbc = bc[0]; udata.xrbc = bc[1]; udata.ylbc = bc[2]; udata.yrbc = bc[3];
  udata.zlbc = bc[4]; udata.zrbc = bc[5];
  udata.gamma = gamma;
  if (udata.SetupDecomp() != 0) return -100;
  for (int v = 0; v < NVAR; ++v) g_force[v] = force ? force[v] : 0.0;

  const long n = nx * ny * nz;
  shim_nvector w{}, wdot{};
  w.nsub = wdot.nsub = (NVAR > 5) ? 6 : 5;
  for (int v = 0; v < w.nsub; ++v) {
    w.sub[v] = fields[v];
    wdot.sub[v] = out[v];
    w.len[v] = wdot.len[v] = (v < 5) ? n : n * (NVAR - 5);
  }
  double t0 = MPI_Wtime();
  int ret = fEuler(t, &w, &wdot, &udata);
  if (seconds) *seconds = MPI_Wtime() - t0;
  return ret;
}

/* ---- chemistry ---- */
static cvklu_data* g_chem = nullptr;
static long g_ncells = 0;

int ref_chem_setup(const char* table_file, long ncells, const double* scale, double current_z) {
  if (g_chem) { cvklu_free_data(g_chem, nullptr); g_chem = nullptr; }
  g_chem = cvklu_setup_data(MPI_COMM_WORLD, table_file, ncells, nullptr, current_z);
  if (!g_chem) return -1;
  g_ncells = ncells;
  for (long i = 0; i < NSPECIES * ncells; ++i) {
    g_chem->scale[i] = scale[i];
    g_chem->inv_scale[i] = 1.0 / scale[i];
  }
  setting_up_extra_variables(g_chem, ncells);
  return 0;
}

void ref_chem_get_state(double* Ts, double* dTs_ge, double* mdens, double* cie, double* h2) {
  for (long i = 0; i < g_ncells; ++i) {
    if (Ts) Ts[i] = g_chem->Ts[i];
    if (dTs_ge) dTs_ge[i] = g_chem->dTs_ge[i];
    if (mdens) mdens[i] = g_chem->mdensity[i];
    if (cie) cie[i] = g_chem->cie_optical_depth_approx[i];
    if (h2) h2[i] = g_chem->h2_optical_depth_approx[i];
  }
}

void ref_chem_set_Ts(const double* Ts) {
  for (long i = 0; i < g_ncells; ++i) g_chem->Ts[i] = Ts[i];
}

int ref_chem_rhs(double t, double* y, double* ydot, double* seconds) {
  shim_nvector Y{}, Yd{};
  Y.nsub = Yd.nsub = 1;
  Y.sub[0] = y; Yd.sub[0] = ydot;
  Y.len[0] = Yd.len[0] = NSPECIES * g_ncells;
  double t0 = MPI_Wtime();
  int ret = calculate_rhs_cvklu(t, &Y, &Yd, g_ncells, g_chem);
  if (seconds) *seconds = MPI_Wtime() - t0;
  return ret;
}

/* Jacobian into dense column-major 10x10 blocks, J[blk*100 + col*10 + row]
 * (the device layout DENSEIDX of src/raja_primordial_network.cpp:40). */
int ref_chem_jac(double t, double* y, double* Jdense, double* seconds) {
  const long nnz = 64 * g_ncells;
  std::vector<double> data(nnz);
  std::vector<sunindextype> rowptrs(NSPECIES * g_ncells + 1), colvals(nnz);
  shim_sunmatrix J{NSPECIES * g_ncells, nnz, data.data(), rowptrs.data(), colvals.data()};
  shim_nvector Y{};
  Y.nsub = 1; Y.sub[0] = y; Y.len[0] = NSPECIES * g_ncells;
  double t0 = MPI_Wtime();
  int ret = calculate_jacobian_cvklu(t, &Y, &Y, &J, g_ncells, g_chem, &Y, &Y, &Y);
  if (seconds) *seconds = MPI_Wtime() - t0;
  for (long i = 0; i < 100 * g_ncells; ++i) Jdense[i] = 0.0;
  for (long r = 0; r < NSPECIES * g_ncells; ++r) {
    const long blk = r / NSPECIES, row = r % NSPECIES;
    for (sunindextype p = rowptrs[r]; p < rowptrs[r + 1]; ++p) {
      const long col = colvals[p] - blk * NSPECIES;
      Jdense[blk * 100 + col * 10 + row] = data[p];
    }
  }
  return ret;
}

}  // extern "C"
