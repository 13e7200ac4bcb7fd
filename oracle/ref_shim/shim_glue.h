/* Declarations for compiling the reference's main programs on one rank (test infrastructure
 * only): the ARKStep / MRIStep / SUNLinearSolver / N_Vector calls they make.  The definitions
 * (oracle/ref_shim/shim_glue.c) abort if called: only the main programs' callbacks run. */
#ifndef GBMV_SHIM_GLUE_H
#define GBMV_SHIM_GLUE_H
#include "shim_core.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef int (*ARKRhsFn)(realtype, N_Vector, N_Vector, void*);
#define ARK_NORMAL 1
#define ARK_SUCCESS 0
#define SUNDIALS_NVEC_MPIMANYVECTOR 14
#define SUNDIALS_NVEC_MANYVECTOR 13
#define SUNLS_SUCCESS 0
#define SUNLS_MEM_FAIL (-803)
#define SUNLS_MEM_NULL (-801)
#define SUNLS_LUFACT_FAIL 808
#define CSR_MAT 1
#define CSC_MAT 0
typedef enum { SUNLINEARSOLVER_DIRECT, SUNLINEARSOLVER_ITERATIVE } SUNLinearSolver_Type;
typedef struct _generic_SUNLinearSolver* SUNLinearSolver;
struct _generic_SUNLinearSolver_Ops {
  SUNLinearSolver_Type (*gettype)(SUNLinearSolver);
  int (*initialize)(SUNLinearSolver);
  int (*setup)(SUNLinearSolver, SUNMatrix);
  int (*solve)(SUNLinearSolver, SUNMatrix, N_Vector, N_Vector, realtype);
  sunindextype (*lastflag)(SUNLinearSolver);
  int (*free)(SUNLinearSolver);
};
struct _generic_SUNLinearSolver {
  void* content;
  struct _generic_SUNLinearSolver_Ops* ops;
  SUNContext sunctx;
};
int N_VGetVectorID(N_Vector v);
sunindextype N_VGetNumSubvectors_ManyVector(N_Vector v);
sunindextype N_VGetNumSubvectors_MPIManyVector(N_Vector v);
N_Vector N_VGetSubvector_ManyVector(N_Vector v, sunindextype k);
void N_VScale(realtype c, N_Vector x, N_Vector z);
void N_VDestroy(N_Vector v);
N_Vector N_VClone(N_Vector v);
N_Vector N_VNew_Serial(sunindextype n, ...);
int N_VEnableFusedOps_Serial(N_Vector v, int on);
int N_VEnableFusedOps_MPIManyVector(N_Vector v, int on);
N_Vector N_VMake_MPIManyVector(MPI_Comm comm, sunindextype n, N_Vector* v, ...);
SUNLinearSolver SUNLinSolNewEmpty(SUNContext ctx);
int SUNLinSolFree(SUNLinearSolver S);
int SUNLinSolInitialize(SUNLinearSolver S);
int SUNLinSolSetup(SUNLinearSolver S, SUNMatrix A);
int SUNLinSolSolve(SUNLinearSolver S, SUNMatrix A, N_Vector x, N_Vector b, realtype tol);
SUNLinearSolver SUNLinSol_KLU(N_Vector y, SUNMatrix A, ...);
SUNMatrix SUNSparseMatrix(sunindextype m, sunindextype n, sunindextype nnz, int type, ...);
sunindextype SUNSparseMatrix_NNZ(SUNMatrix A);
void SUNMatDestroy(SUNMatrix A);
void* ARKStepCreate(ARKRhsFn fe, ARKRhsFn fi, realtype t0, N_Vector y0, ...);
void ARKStepFree(void** mem);
int ARKStepEvolve(void* mem, realtype tout, N_Vector y, realtype* t, int task);
int ARKStepSetUserData(void* mem, void* ud);
int ARKStepSetTableNum(void* mem, int itable, int etable);
int ARKStepSetStabilityFn(void* mem, ...);
int ARKStepSetSafetyFactor(void* mem, realtype v);
int ARKStepSetPredictorMethod(void* mem, int v);
int ARKStepSetPostprocessStepFn(void* mem, ...);
int ARKStepSetNonlinConvCoef(void* mem, realtype v);
int ARKStepSetMinStep(void* mem, realtype v);
int ARKStepSetMaxStep(void* mem, realtype v);
int ARKStepSetMaxNumSteps(void* mem, long v);
int ARKStepSetMaxNonlinIters(void* mem, int v);
int ARKStepSetMaxHnilWarns(void* mem, int v);
int ARKStepSetMaxGrowth(void* mem, realtype v);
int ARKStepSetMaxFirstGrowth(void* mem, realtype v);
int ARKStepSetMaxErrTestFails(void* mem, int v);
int ARKStepSetMaxEFailGrowth(void* mem, realtype v);
int ARKStepSetLinearSolver(void* mem, SUNLinearSolver LS, SUNMatrix A);
int ARKStepSetJacFn(void* mem, ...);
int ARKStepSetInitStep(void* mem, realtype v);
int ARKStepSetErrorBias(void* mem, realtype v);
int ARKStepSetDiagnostics(void* mem, FILE* f);
int ARKStepSetDenseOrder(void* mem, int v);
int ARKStepSetAdaptivityMethod(void* mem, int imethod, int idefault, int pq, realtype* adapt);
int ARKStepSVtolerances(void* mem, realtype rtol, N_Vector atol);
int ARKStepSetStopTime(void* mem, realtype t);
int ARKStepSetFixedStep(void* mem, realtype h);
int ARKStepGetNumSteps(void* mem, long* n);
int ARKStepGetNumStepAttempts(void* mem, long* n);
int ARKStepGetNumRhsEvals(void* mem, long* nfe, long* nfi);
int ARKStepGetNumLinSolvSetups(void* mem, long* n);
int ARKStepGetNumLinIters(void* mem, long* n);
int ARKStepGetNumLinConvFails(void* mem, long* n);
int ARKStepGetNumJacEvals(void* mem, long* n);
int ARKStepGetNumErrTestFails(void* mem, long* n);
int ARKStepGetNonlinSolvStats(void* mem, long* nni, long* ncf);
int ARKStepGetLastStep(void* mem, realtype* h);
#ifdef __cplusplus
}
#endif
#endif
