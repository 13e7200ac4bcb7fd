// ARKODE-signature callbacks over the gbmv C ABI (see gbmv_arkode.h).  Each body takes the
// device pointers of the MPIManyVector's components and makes one drop-in call.
#include "gbmv_arkode.h"

#include <stdlib.h>

#include <nvector/nvector_mpimanyvector.h>
#include <sunmatrix/sunmatrix_magmadense.h>

namespace {

// Device pointers of the (up to) six components; components absent from the vector (the
// chemistry of a pure-hydrodynamics run) are null.  Returns false if a present component
// has no device data.
bool components(N_Vector v, double* p[6]) {
  if (!v) return false;
  const sunindextype n = N_VGetNumSubvectors_MPIManyVector(v);
  for (int k = 0; k < 6; ++k) {
    p[k] = nullptr;
    if (k >= n) continue;
    N_Vector s = N_VGetSubvector_MPIManyVector(v, k);
    if (!s) return false;
    p[k] = N_VGetDeviceArrayPointer(s);
    if (!p[k]) return false;
  }
  return true;
}

// forcing vectors of the MRI inner problem as 6 device pointers each
bool forcing_pointers(N_Vector* forcing, int nforcing, const double* fp[8 * 6]) {
  if (nforcing > 8) return false;
  for (int i = 0; i < nforcing; ++i) {
    double* p[6];
    if (!components(forcing[i], p)) return false;
    for (int k = 0; k < 6; ++k) fp[6 * i + k] = p[k];
  }
  return true;
}

struct BlockLSContent {
  gbmv_block_ls ls;
  sunindextype subvec;
  gbmv_arkode_data* data;
  int last_flag;
};

BlockLSContent* content(SUNLinearSolver S) { return static_cast<BlockLSContent*>(S->content); }

SUNLinearSolver_Type block_gettype(SUNLinearSolver) { return SUNLINEARSOLVER_DIRECT; }

int block_initialize(SUNLinearSolver S) {
  content(S)->last_flag = SUNLS_SUCCESS;
  return SUNLS_SUCCESS;
}

// A = I - gamma J formed by ARKLS in the block matrix: factor every block in place
int block_setup(SUNLinearSolver S, SUNMatrix A) {
  BlockLSContent* c = content(S);
  const int rc = gbmv_block_ls_setup(c->ls, SUNMatrix_MagmaDense_Data(A), c->data->stream);
  c->last_flag = rc == 0 ? SUNLS_SUCCESS : (rc > 0 ? SUNLS_LUFACT_FAIL : SUNLS_PACKAGE_FAIL_UNREC);
  return c->last_flag;
}

// x = A^{-1} b on the chemistry subvector (the direct solve ignores tol)
int block_solve(SUNLinearSolver S, SUNMatrix A, N_Vector x, N_Vector b, realtype) {
  BlockLSContent* c = content(S);
  N_Vector xs = N_VGetSubvector_MPIManyVector(x, c->subvec);
  N_Vector bs = N_VGetSubvector_MPIManyVector(b, c->subvec);
  if (!xs || !bs) {
    c->last_flag = SUNLS_MEM_FAIL;
    return c->last_flag;
  }
  const int rc = gbmv_block_ls_solve(c->ls, SUNMatrix_MagmaDense_Data(A),
                                     N_VGetDeviceArrayPointer(bs), N_VGetDeviceArrayPointer(xs),
                                     c->data->stream);
  c->last_flag = rc == 0 ? SUNLS_SUCCESS : SUNLS_PACKAGE_FAIL_UNREC;
  return c->last_flag;
}

sunindextype block_lastflag(SUNLinearSolver S) { return content(S)->last_flag; }

int block_free(SUNLinearSolver S) {
  if (!S) return SUNLS_SUCCESS;
  if (S->content) {
    gbmv_block_ls_destroy(content(S)->ls);
    free(S->content);
    S->content = nullptr;
  }
  SUNLinSolFreeEmpty(S);
  return SUNLS_SUCCESS;
}

int fast_evolve(gbmv_inner_content* ic, realtype t0, realtype tout, N_Vector y) {
  double* w[6];
  if (!components(y, w)) return -1;
  realtype tshift = 0.0, tscale = 1.0;
  N_Vector* forcing = nullptr;
  int nforcing = 0;
  if (MRIStepInnerStepper_GetForcingData(ic->stepper, &tshift, &tscale, &forcing, &nforcing))
    return -1;
  const double* fp[8 * 6];
  if (!forcing_pointers(forcing, nforcing, fp)) return -1;
  gbmv_arkode_data* d = ic->data;
  const int nfail = gbmv_mri_fast_evolve(d->hydro, d->chem, t0, tout, w, d->time_units,
                                         nforcing, nforcing ? fp : nullptr, tshift, tscale,
                                         &d->fast_opts, nullptr, d->stream);
  // failed cells are a recoverable failure: MRIStep retries with a smaller slow step
  return nfail < 0 ? nfail : (nfail > 0 ? 1 : 0);
}

}  // namespace

extern "C" {

int gbmv_ark_feuler(realtype t, N_Vector w, N_Vector wdot, void* user_data) {
  gbmv_arkode_data* d = static_cast<gbmv_arkode_data*>(user_data);
  double *pw[6], *pd[6];
  if (!d || !components(w, pw) || !components(wdot, pd)) return -1;
  return gbmv_feuler(d->hydro, t, pw, pd, d->precision, d->stream);
}

int gbmv_ark_fexpl(realtype t, N_Vector w, N_Vector wdot, void* user_data) {
  gbmv_arkode_data* d = static_cast<gbmv_arkode_data*>(user_data);
  double *pw[6], *pd[6];
  if (!d || !components(w, pw) || !components(wdot, pd)) return -1;
  return gbmv_fexpl(d->hydro, d->chem, t, pw, pd, d->energy_units, d->precision, d->stream);
}

int gbmv_ark_fimpl(realtype t, N_Vector w, N_Vector wdot, void* user_data) {
  gbmv_arkode_data* d = static_cast<gbmv_arkode_data*>(user_data);
  double *pw[6], *pd[6];
  if (!d || !components(w, pw) || !components(wdot, pd)) return -1;
  // the fast right-hand side without forcing is exactly fimpl: fluid 0, TimeUnits x source
  return gbmv_ffast(d->hydro, d->chem, t, pw, pd, d->time_units, 0, nullptr, 0.0, 1.0,
                    d->stream);
}

int gbmv_ark_ffast(realtype t, N_Vector w, N_Vector wdot, void* user_data) {
  gbmv_inner_content* ic = static_cast<gbmv_inner_content*>(user_data);
  double *pw[6], *pd[6];
  if (!ic || !ic->data || !components(w, pw) || !components(wdot, pd)) return -1;
  realtype tshift = 0.0, tscale = 1.0;
  N_Vector* forcing = nullptr;
  int nforcing = 0;
  if (!ic->disable_forcing &&
      MRIStepInnerStepper_GetForcingData(ic->stepper, &tshift, &tscale, &forcing, &nforcing))
    return -1;
  const double* fp[8 * 6];
  if (!forcing_pointers(forcing, nforcing, fp)) return -1;
  gbmv_arkode_data* d = ic->data;
  return gbmv_ffast(d->hydro, d->chem, t, pw, pd, d->time_units, nforcing,
                    nforcing ? fp : nullptr, tshift, tscale, d->stream);
}

int gbmv_ark_jac(realtype t, N_Vector w, N_Vector, SUNMatrix J, void* user_data, N_Vector,
                 N_Vector, N_Vector) {
  gbmv_arkode_data* d = static_cast<gbmv_arkode_data*>(user_data);
  double* pw[6];
  if (!d || !components(w, pw) || !pw[5]) return -1;
  return gbmv_chem_jac(d->chem, t, pw[5], SUNMatrix_MagmaDense_Data(J), d->time_units,
                       d->stream);
}

int gbmv_ark_postprocess(realtype, N_Vector w, void* user_data) {
  gbmv_arkode_data* d = static_cast<gbmv_arkode_data*>(user_data);
  double* pw[6];
  if (!d || !components(w, pw)) return -1;
  return gbmv_postprocess_step(d->hydro, d->chem, pw, d->energy_units, d->stream);
}

int gbmv_ark_stability(N_Vector w, realtype, realtype* dt_stab, void* user_data) {
  gbmv_arkode_data* d = static_cast<gbmv_arkode_data*>(user_data);
  double* pw[6];
  if (!d || !dt_stab || !components(w, pw)) return -1;
  return gbmv_stability(d->hydro, pw, d->cfl, dt_stab, d->stream);
}

SUNLinearSolver gbmv_SUNLinSol_Block(N_Vector x, sunindextype subvec, gbmv_arkode_data* data,
                                     SUNContext ctx) {
  if (!x || !data || subvec >= N_VGetNumSubvectors_MPIManyVector(x)) return nullptr;
  N_Vector xs = N_VGetSubvector_MPIManyVector(x, subvec);
  if (!xs) return nullptr;
  const long nblocks = (long)(N_VGetLength(xs) / 10);
  SUNLinearSolver S = SUNLinSolNewEmpty(ctx);
  if (!S) return nullptr;
  BlockLSContent* c = static_cast<BlockLSContent*>(malloc(sizeof(BlockLSContent)));
  if (!c || gbmv_block_ls_create(nblocks, &c->ls) != GBMV_OK) {
    free(c);
    SUNLinSolFreeEmpty(S);
    return nullptr;
  }
  c->subvec = subvec;
  c->data = data;
  c->last_flag = SUNLS_SUCCESS;
  S->content = c;
  S->ops->gettype = block_gettype;
  S->ops->initialize = block_initialize;
  S->ops->setup = block_setup;
  S->ops->solve = block_solve;
  S->ops->lastflag = block_lastflag;
  S->ops->free = block_free;
  return S;
}

int gbmv_inner_evolve(MRIStepInnerStepper stepper, realtype t0, realtype tout, N_Vector y) {
  void* c = nullptr;
  if (MRIStepInnerStepper_GetContent(stepper, &c) || !c) return -1;
  return fast_evolve(static_cast<gbmv_inner_content*>(c), t0, tout, y);
}

int gbmv_inner_fullrhs(MRIStepInnerStepper stepper, realtype t, N_Vector y, N_Vector f, int) {
  void* c = nullptr;
  if (MRIStepInnerStepper_GetContent(stepper, &c) || !c) return -1;
  gbmv_inner_content* ic = static_cast<gbmv_inner_content*>(c);
  const int keep = ic->disable_forcing;
  ic->disable_forcing = 1;  // the full right-hand side of the fast problem, without forcing
  const int rc = gbmv_ark_ffast(t, y, f, ic);
  ic->disable_forcing = keep;
  return rc;
}

int gbmv_inner_reset(MRIStepInnerStepper, realtype, N_Vector) {
  return 0;  // the per-cell DIRK starts every evolve afresh: no history to reset
}

}  // extern "C"
