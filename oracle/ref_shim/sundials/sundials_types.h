/* Stand-in header: forwards to the one-rank shim (test infrastructure only). */
#ifndef GBMV_SHIM_SUNDIALS_SUNDIALS_TYPES_H
#define GBMV_SHIM_SUNDIALS_SUNDIALS_TYPES_H
#include <math.h>
#include "../shim_core.h"
#endif
