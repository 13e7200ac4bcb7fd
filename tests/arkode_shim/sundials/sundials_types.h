/* Test stand-in for SUNDIALS 6's sundials_types.h: only what the ARKODE adapter
 * (sundials-manyvector-demo_gb300/adapter) uses.  TEST INFRASTRUCTURE ONLY. */
#ifndef SHIM_SUNDIALS_TYPES_H
#define SHIM_SUNDIALS_TYPES_H
typedef double realtype;
typedef long sunindextype;
typedef int booleantype;
typedef struct shim_context* SUNContext;
#endif
