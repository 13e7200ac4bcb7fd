/* Stand-in header: forwards to the one-rank shim (test infrastructure only). */
#ifndef GBMV_SHIM_SUNLINSOL_SUNLINSOL_KLU_H
#define GBMV_SHIM_SUNLINSOL_SUNLINSOL_KLU_H
#include <math.h>
#include "../shim_core.h"
#endif
