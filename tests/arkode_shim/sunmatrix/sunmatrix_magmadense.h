/* Test stand-in for SUNDIALS 6's SUNMATRIX_MAGMADENSE data accessor.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef SHIM_SUNMATRIX_MAGMADENSE_H
#define SHIM_SUNMATRIX_MAGMADENSE_H
#include <sundials/sundials_matrix.h>
#ifdef __cplusplus
extern "C" {
#endif
realtype* SUNMatrix_MagmaDense_Data(SUNMatrix A);
#ifdef __cplusplus
}
#endif
#endif
