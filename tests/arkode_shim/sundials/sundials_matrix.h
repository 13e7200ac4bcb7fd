/* Test stand-in for SUNDIALS 6's generic SUNMatrix.  TEST INFRASTRUCTURE ONLY. */
#ifndef SHIM_SUNDIALS_MATRIX_H
#define SHIM_SUNDIALS_MATRIX_H
#include "sundials_types.h"
typedef struct shim_sunmatrix* SUNMatrix;
struct shim_sunmatrix {
  double* data;          /* device blocks, 10 x 10 column-major each */
  sunindextype nblocks;
};
#endif
