/* Stand-in header: forwards to the one-rank shim (test infrastructure only). */
#ifndef GBMV_SHIM_ARKODE_ARKODE_BUTCHER_DIRK_H
#define GBMV_SHIM_ARKODE_ARKODE_BUTCHER_DIRK_H
#include <math.h>
#include "../shim_core.h"
#endif
