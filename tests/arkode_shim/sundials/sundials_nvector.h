/* Test stand-in for SUNDIALS 6's generic N_Vector (sundials_nvector.h): a ManyVector of
 * device arrays.  TEST INFRASTRUCTURE ONLY. */
#ifndef SHIM_SUNDIALS_NVECTOR_H
#define SHIM_SUNDIALS_NVECTOR_H
#include "sundials_types.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct shim_nvector* N_Vector;
struct shim_nvector {
  int nsub;            /* > 0: a ManyVector of nsub subvectors; 0: a plain device array */
  N_Vector sub[8];
  double* data;        /* device data of a plain vector */
  sunindextype length;
};
realtype* N_VGetDeviceArrayPointer(N_Vector v);
sunindextype N_VGetLength(N_Vector v);
#ifdef __cplusplus
}
#endif
#endif
