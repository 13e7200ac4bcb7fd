// Test harness for the ARKODE adapter (sundials-manyvector-demo_gb300/adapter): the stand-in
// SUNDIALS functions the adapter calls, and extern "C" drivers that wrap device arrays into
// stand-in MPIManyVectors / block matrices / inner steppers and call the adapter's callbacks
// exactly as ARKStep and MRIStep would.  TEST INFRASTRUCTURE ONLY.
#include <stdlib.h>
#include <string.h>

#include <arkode/arkode_mristep.h>
#include <nvector/nvector_mpimanyvector.h>
#include <sundials/sundials_linearsolver.h>
#include <sunmatrix/sunmatrix_magmadense.h>

#include "gbmv_arkode.h"

extern "C" {

// ---- stand-in SUNDIALS functions
realtype* N_VGetDeviceArrayPointer(N_Vector v) { return v && v->nsub == 0 ? v->data : nullptr; }
sunindextype N_VGetLength(N_Vector v) {
  if (!v) return 0;
  if (v->nsub == 0) return v->length;
  sunindextype n = 0;
  for (int k = 0; k < v->nsub; ++k) n += N_VGetLength(v->sub[k]);
  return n;
}
N_Vector N_VGetSubvector_MPIManyVector(N_Vector v, sunindextype k) {
  return (v && k >= 0 && k < v->nsub) ? v->sub[k] : nullptr;
}
sunindextype N_VGetNumSubvectors_MPIManyVector(N_Vector v) { return v ? v->nsub : 0; }
realtype* SUNMatrix_MagmaDense_Data(SUNMatrix A) { return A ? A->data : nullptr; }
SUNLinearSolver SUNLinSolNewEmpty(SUNContext ctx) {
  SUNLinearSolver S = static_cast<SUNLinearSolver>(calloc(1, sizeof(*S)));
  if (!S) return nullptr;
  S->ops = static_cast<SUNLinearSolver_Ops>(calloc(1, sizeof(*S->ops)));
  if (!S->ops) { free(S); return nullptr; }
  S->sunctx = ctx;
  return S;
}
void SUNLinSolFreeEmpty(SUNLinearSolver S) {
  if (!S) return;
  free(S->ops);
  free(S);
}
int MRIStepInnerStepper_GetContent(MRIStepInnerStepper s, void** c) {
  if (!s || !c) return -1;
  *c = s->content;
  return 0;
}
int MRIStepInnerStepper_GetForcingData(MRIStepInnerStepper s, realtype* tshift,
                                       realtype* tscale, N_Vector** forcing, int* nforcing) {
  if (!s) return -1;
  *tshift = s->tshift;
  *tscale = s->tscale;
  *forcing = s->forcing;
  *nforcing = s->nforcing;
  return 0;
}

}  // extern "C"

namespace {

// a ManyVector over ncomp device arrays (lengths in doubles)
struct MV {
  shim_nvector top{};
  shim_nvector comp[6]{};
  MV(double* const* p, const long* len, int ncomp) {
    top.nsub = ncomp;
    for (int k = 0; k < ncomp; ++k) {
      comp[k].nsub = 0;
      comp[k].data = p[k];
      comp[k].length = len[k];
      top.sub[k] = &comp[k];
    }
  }
  N_Vector v() { return &top; }
};

gbmv_arkode_data g_data;

}  // namespace

extern "C" {

int drv_setup(void* hydro, void* chem, double eu, double tu, double cfl, int precision,
              void* stream, const gbmv_dirk_opts* fast) {
  memset(&g_data, 0, sizeof g_data);
  g_data.hydro = static_cast<gbmv_hydro>(hydro);
  g_data.chem = static_cast<gbmv_chem>(chem);
  g_data.energy_units = eu;
  g_data.time_units = tu;
  g_data.cfl = cfl;
  g_data.precision = precision;
  g_data.stream = stream;
  if (fast) g_data.fast_opts = *fast;
  else gbmv_dirk_opts_default(&g_data.fast_opts);
  return 0;
}

// which: 0 fEuler, 1 fexpl, 2 fimpl
int drv_rhs(int which, double t, double* const* w, double* const* wdot, const long* len,
            int ncomp) {
  MV a(w, len, ncomp), b(wdot, len, ncomp);
  switch (which) {
    case 0: return gbmv_ark_feuler(t, a.v(), b.v(), &g_data);
    case 1: return gbmv_ark_fexpl(t, a.v(), b.v(), &g_data);
    case 2: return gbmv_ark_fimpl(t, a.v(), b.v(), &g_data);
    default: return -1;
  }
}

// ffast with the MRI forcing (nforcing vectors of 6 components, row-major pointers)
int drv_ffast(double t, double* const* w, double* const* wdot, const long* len, int nforcing,
              double* const* forcing, double tshift, double tscale) {
  MV a(w, len, 6), b(wdot, len, 6);
  MV* f[8];
  N_Vector fv[8];
  for (int i = 0; i < nforcing; ++i) {
    f[i] = new MV(forcing + 6 * i, len, 6);
    fv[i] = f[i]->v();
  }
  shim_inner_stepper st{nullptr, tshift, tscale, fv, nforcing};
  gbmv_inner_content ic{&g_data, &st, 0};
  st.content = &ic;
  const int rc = gbmv_ark_ffast(t, a.v(), b.v(), &ic);
  for (int i = 0; i < nforcing; ++i) delete f[i];
  return rc;
}

int drv_jac(double t, double* const* w, const long* len, double* J, long nblocks) {
  MV a(w, len, 6);
  shim_sunmatrix M{J, nblocks};
  return gbmv_ark_jac(t, a.v(), a.v(), &M, &g_data, nullptr, nullptr, nullptr);
}

// the block linear solver through its SUNLinearSolver ops: create, initialize, setup on A
// (A = I - gamma J already), solve x = A^{-1} b on subvector 5, free; returns setup's flag
// (or the solve's if setup succeeded)
int drv_linsol(double* const* x, double* const* b, const long* len, double* A, long nblocks) {
  MV xv(x, len, 6), bv(b, len, 6);
  SUNLinearSolver S = gbmv_SUNLinSol_Block(xv.v(), 5, &g_data, nullptr);
  if (!S) return -1000;
  if (S->ops->gettype(S) != SUNLINEARSOLVER_DIRECT) return -1001;
  int rc = S->ops->initialize(S);
  shim_sunmatrix M{A, nblocks};
  if (!rc) rc = S->ops->setup(S, &M);
  if (!rc) rc = S->ops->solve(S, &M, xv.v(), bv.v(), 0.0);
  if (S->ops->lastflag(S) != rc) rc = -1002;
  S->ops->free(S);
  return rc;
}

// the inner stepper: evolve (with forcing), fullrhs, reset
int drv_inner(int which, double t0, double tout, double* const* y, double* const* f,
              const long* len, int nforcing, double* const* forcing, double tshift,
              double tscale) {
  MV yv(y, len, 6);
  MV* fm[8];
  N_Vector fv[8];
  for (int i = 0; i < nforcing; ++i) {
    fm[i] = new MV(forcing + 6 * i, len, 6);
    fv[i] = fm[i]->v();
  }
  shim_inner_stepper st{nullptr, tshift, tscale, fv, nforcing};
  gbmv_inner_content ic{&g_data, &st, 0};
  st.content = &ic;
  int rc = -1;
  if (which == 0) {
    rc = gbmv_inner_evolve(&st, t0, tout, yv.v());
  } else if (which == 1) {
    MV fo(f, len, 6);
    rc = gbmv_inner_fullrhs(&st, t0, yv.v(), fo.v(), 0);
  } else if (which == 2) {
    rc = gbmv_inner_reset(&st, t0, yv.v());
  }
  for (int i = 0; i < nforcing; ++i) delete fm[i];
  return rc;
}

int drv_post(double t, double* const* w, const long* len) {
  MV a(w, len, 6);
  return gbmv_ark_postprocess(t, a.v(), &g_data);
}

int drv_stability(double* const* w, const long* len, int ncomp, double* dt) {
  MV a(w, len, ncomp);
  return gbmv_ark_stability(a.v(), 0.0, dt, &g_data);
}

}  // extern "C"
