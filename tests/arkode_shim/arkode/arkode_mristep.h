/* Test stand-in for SUNDIALS 6's MRIStep inner-stepper interface (content and forcing data
 * access).  TEST INFRASTRUCTURE ONLY. */
#ifndef SHIM_ARKODE_MRISTEP_H
#define SHIM_ARKODE_MRISTEP_H
#include <sundials/sundials_nvector.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct shim_inner_stepper* MRIStepInnerStepper;
struct shim_inner_stepper {
  void* content;
  realtype tshift, tscale;
  N_Vector* forcing;
  int nforcing;
};
int MRIStepInnerStepper_GetContent(MRIStepInnerStepper stepper, void** content);
int MRIStepInnerStepper_GetForcingData(MRIStepInnerStepper stepper, realtype* tshift,
                                       realtype* tscale, N_Vector** forcing, int* nforcing);
#ifdef __cplusplus
}
#endif
#endif
