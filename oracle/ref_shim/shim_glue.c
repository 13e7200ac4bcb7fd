/* Definitions for shim_glue.h (test infrastructure only).  The main programs' own driver
 * calls (ARKStep setup, evolve, statistics, the KLU solver) are never reached when only their
 * callbacks are called: they report and abort.  Subvector access returns views into the
 * ManyVector's component arrays. */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>

#include "shim_glue.h"

static void unreachable(const char* what) {
  fprintf(stderr, "ref shim: %s is not available in this one-rank build\n", what);
  abort();
}

/* a ring of views: each is a one-component vector over component k of its parent */
static struct shim_nvector g_views[64];
static int g_next_view = 0;

N_Vector N_VGetSubvector_MPIManyVector(N_Vector v, sunindextype k) {
  if (!v || k < 0 || k >= v->nsub) return NULL;
  N_Vector s = &g_views[g_next_view];
  g_next_view = (g_next_view + 1) % 64;
  s->nsub = 1;
  s->sub[0] = v->sub[k];
  s->len[0] = v->len[k];
  return s;
}
N_Vector N_VGetSubvector_ManyVector(N_Vector v, sunindextype k) {
  return N_VGetSubvector_MPIManyVector(v, k);
}
sunindextype N_VGetNumSubvectors_ManyVector(N_Vector v) { return v ? v->nsub : 0; }
sunindextype N_VGetNumSubvectors_MPIManyVector(N_Vector v) { return v ? v->nsub : 0; }
int N_VGetVectorID(N_Vector v) { (void)v; return SUNDIALS_NVEC_MPIMANYVECTOR; }
void N_VScale(realtype c, N_Vector x, N_Vector z) {
  for (int s = 0; s < x->nsub; ++s)
    for (long i = 0; i < x->len[s]; ++i) z->sub[s][i] = c * x->sub[s][i];
}
void N_VDestroy(N_Vector v) { (void)v; unreachable("N_VDestroy"); }
N_Vector N_VClone(N_Vector v) { (void)v; unreachable("N_VClone"); return NULL; }
N_Vector N_VNew_Serial(sunindextype n, ...) { (void)n; unreachable("N_VNew_Serial"); return NULL; }
int N_VEnableFusedOps_Serial(N_Vector v, int on) { (void)v; (void)on; return 0; }
int N_VEnableFusedOps_MPIManyVector(N_Vector v, int on) { (void)v; (void)on; return 0; }
N_Vector N_VMake_MPIManyVector(MPI_Comm comm, sunindextype n, N_Vector* v, ...) {
  (void)comm; (void)n; (void)v;
  unreachable("N_VMake_MPIManyVector");
  return NULL;
}
SUNLinearSolver SUNLinSolNewEmpty(SUNContext ctx) { (void)ctx; unreachable("SUNLinSolNewEmpty"); return NULL; }
int SUNLinSolFree(SUNLinearSolver S) { (void)S; unreachable("SUNLinSolFree"); return 0; }
int SUNLinSolInitialize(SUNLinearSolver S) { (void)S; unreachable("SUNLinSolInitialize"); return 0; }
int SUNLinSolSetup(SUNLinearSolver S, SUNMatrix A) { (void)S; (void)A; unreachable("SUNLinSolSetup"); return 0; }
int SUNLinSolSolve(SUNLinearSolver S, SUNMatrix A, N_Vector x, N_Vector b, realtype tol) {
  (void)S; (void)A; (void)x; (void)b; (void)tol;
  unreachable("SUNLinSolSolve");
  return 0;
}
SUNLinearSolver SUNLinSol_KLU(N_Vector y, SUNMatrix A, ...) { (void)y; (void)A; unreachable("SUNLinSol_KLU"); return NULL; }
SUNMatrix SUNSparseMatrix(sunindextype m, sunindextype n, sunindextype nnz, int type, ...) {
  (void)m; (void)n; (void)nnz; (void)type;
  unreachable("SUNSparseMatrix");
  return NULL;
}
sunindextype SUNSparseMatrix_NNZ(SUNMatrix A) { return A ? A->nnz : 0; }
void SUNMatDestroy(SUNMatrix A) { (void)A; unreachable("SUNMatDestroy"); }
void* ARKStepCreate(ARKRhsFn fe, ARKRhsFn fi, realtype t0, N_Vector y0, ...) {
  (void)fe; (void)fi; (void)t0; (void)y0;
  unreachable("ARKStepCreate");
  return NULL;
}
void ARKStepFree(void** mem) { (void)mem; unreachable("ARKStepFree"); }

int ARKStepEvolve(void* mem, realtype tout, N_Vector y, realtype* t, int task) {
  (void)mem; (void)tout; (void)y; (void)t; (void)task; unreachable("ARKStepEvolve"); return 0;
}
int ARKStepSetUserData(void* mem, void* ud) { (void)mem; (void)ud; unreachable("ARKStepSetUserData"); return 0; }
int ARKStepSetTableNum(void* mem, int a, int b) { (void)mem; (void)a; (void)b; unreachable("ARKStepSetTableNum"); return 0; }
int ARKStepSetStabilityFn(void* mem, ...) { (void)mem; unreachable("ARKStepSetStabilityFn"); return 0; }
int ARKStepSetSafetyFactor(void* mem, realtype v) { (void)mem; (void)v; unreachable("ARKStepSetSafetyFactor"); return 0; }
int ARKStepSetPredictorMethod(void* mem, int v) { (void)mem; (void)v; unreachable("ARKStepSetPredictorMethod"); return 0; }
int ARKStepSetPostprocessStepFn(void* mem, ...) { (void)mem; unreachable("ARKStepSetPostprocessStepFn"); return 0; }
int ARKStepSetNonlinConvCoef(void* mem, realtype v) { (void)mem; (void)v; unreachable("ARKStepSetNonlinConvCoef"); return 0; }
int ARKStepSetMinStep(void* mem, realtype v) { (void)mem; (void)v; unreachable("ARKStepSetMinStep"); return 0; }
int ARKStepSetMaxStep(void* mem, realtype v) { (void)mem; (void)v; unreachable("ARKStepSetMaxStep"); return 0; }
int ARKStepSetMaxNumSteps(void* mem, long v) { (void)mem; (void)v; unreachable("ARKStepSetMaxNumSteps"); return 0; }
int ARKStepSetMaxNonlinIters(void* mem, int v) { (void)mem; (void)v; unreachable("ARKStepSetMaxNonlinIters"); return 0; }
int ARKStepSetMaxHnilWarns(void* mem, int v) { (void)mem; (void)v; unreachable("ARKStepSetMaxHnilWarns"); return 0; }
int ARKStepSetMaxGrowth(void* mem, realtype v) { (void)mem; (void)v; unreachable("ARKStepSetMaxGrowth"); return 0; }
int ARKStepSetMaxFirstGrowth(void* mem, realtype v) { (void)mem; (void)v; unreachable("ARKStepSetMaxFirstGrowth"); return 0; }
int ARKStepSetMaxErrTestFails(void* mem, int v) { (void)mem; (void)v; unreachable("ARKStepSetMaxErrTestFails"); return 0; }
int ARKStepSetMaxEFailGrowth(void* mem, realtype v) { (void)mem; (void)v; unreachable("ARKStepSetMaxEFailGrowth"); return 0; }
int ARKStepSetLinearSolver(void* mem, SUNLinearSolver LS, SUNMatrix A) { (void)mem; (void)LS; (void)A; unreachable("ARKStepSetLinearSolver"); return 0; }
int ARKStepSetJacFn(void* mem, ...) { (void)mem; unreachable("ARKStepSetJacFn"); return 0; }
int ARKStepSetInitStep(void* mem, realtype v) { (void)mem; (void)v; unreachable("ARKStepSetInitStep"); return 0; }
int ARKStepSetErrorBias(void* mem, realtype v) { (void)mem; (void)v; unreachable("ARKStepSetErrorBias"); return 0; }
int ARKStepSetDiagnostics(void* mem, FILE* f) { (void)mem; (void)f; unreachable("ARKStepSetDiagnostics"); return 0; }
int ARKStepSetDenseOrder(void* mem, int v) { (void)mem; (void)v; unreachable("ARKStepSetDenseOrder"); return 0; }
int ARKStepSetAdaptivityMethod(void* mem, int a, int b, int c, realtype* d) { (void)mem; (void)a; (void)b; (void)c; (void)d; unreachable("ARKStepSetAdaptivityMethod"); return 0; }
int ARKStepSVtolerances(void* mem, realtype r, N_Vector a) { (void)mem; (void)r; (void)a; unreachable("ARKStepSVtolerances"); return 0; }
int ARKStepSetStopTime(void* mem, realtype t) { (void)mem; (void)t; unreachable("ARKStepSetStopTime"); return 0; }
int ARKStepSetFixedStep(void* mem, realtype h) { (void)mem; (void)h; unreachable("ARKStepSetFixedStep"); return 0; }
int ARKStepGetNumSteps(void* mem, long* n) { (void)mem; (void)n; unreachable("ARKStepGetNumSteps"); return 0; }
int ARKStepGetNumStepAttempts(void* mem, long* n) { (void)mem; (void)n; unreachable("ARKStepGetNumStepAttempts"); return 0; }
int ARKStepGetNumRhsEvals(void* mem, long* a, long* b) { (void)mem; (void)a; (void)b; unreachable("ARKStepGetNumRhsEvals"); return 0; }
int ARKStepGetNumLinSolvSetups(void* mem, long* n) { (void)mem; (void)n; unreachable("ARKStepGetNumLinSolvSetups"); return 0; }
int ARKStepGetNumLinIters(void* mem, long* n) { (void)mem; (void)n; unreachable("ARKStepGetNumLinIters"); return 0; }
int ARKStepGetNumLinConvFails(void* mem, long* n) { (void)mem; (void)n; unreachable("ARKStepGetNumLinConvFails"); return 0; }
int ARKStepGetNumJacEvals(void* mem, long* n) { (void)mem; (void)n; unreachable("ARKStepGetNumJacEvals"); return 0; }
int ARKStepGetNumErrTestFails(void* mem, long* n) { (void)mem; (void)n; unreachable("ARKStepGetNumErrTestFails"); return 0; }
int ARKStepGetNonlinSolvStats(void* mem, long* a, long* b) { (void)mem; (void)a; (void)b; unreachable("ARKStepGetNonlinSolvStats"); return 0; }
int ARKStepGetLastStep(void* mem, realtype* h) { (void)mem; (void)h; unreachable("ARKStepGetLastStep"); return 0; }
