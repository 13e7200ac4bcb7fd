/* Test stand-in for SUNDIALS 6's generic SUNLinearSolver (the struct, its ops table, the
 * empty constructor / destructor and the return codes the adapter uses).
 * TEST INFRASTRUCTURE ONLY. */
#ifndef SHIM_SUNDIALS_LINEARSOLVER_H
#define SHIM_SUNDIALS_LINEARSOLVER_H
#include "sundials_matrix.h"
#include "sundials_nvector.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef enum {
  SUNLINEARSOLVER_DIRECT,
  SUNLINEARSOLVER_ITERATIVE,
  SUNLINEARSOLVER_MATRIX_ITERATIVE,
  SUNLINEARSOLVER_MATRIX_EMBEDDED
} SUNLinearSolver_Type;
#define SUNLS_SUCCESS 0
#define SUNLS_MEM_FAIL (-803)
#define SUNLS_PACKAGE_FAIL_UNREC (-809)
#define SUNLS_LUFACT_FAIL 808
typedef struct _generic_SUNLinearSolver* SUNLinearSolver;
typedef struct _generic_SUNLinearSolver_Ops* SUNLinearSolver_Ops;
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
  SUNLinearSolver_Ops ops;
  SUNContext sunctx;
};
SUNLinearSolver SUNLinSolNewEmpty(SUNContext sunctx);
void SUNLinSolFreeEmpty(SUNLinearSolver S);
#ifdef __cplusplus
}
#endif
#endif
