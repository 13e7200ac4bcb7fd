/* Test stand-in for SUNDIALS 6's MPIManyVector accessors.  TEST INFRASTRUCTURE ONLY. */
#ifndef SHIM_NVECTOR_MPIMANYVECTOR_H
#define SHIM_NVECTOR_MPIMANYVECTOR_H
#include <sundials/sundials_nvector.h>
#ifdef __cplusplus
extern "C" {
#endif
N_Vector N_VGetSubvector_MPIManyVector(N_Vector v, sunindextype vec_num);
sunindextype N_VGetNumSubvectors_MPIManyVector(N_Vector v);
#ifdef __cplusplus
}
#endif
#endif
