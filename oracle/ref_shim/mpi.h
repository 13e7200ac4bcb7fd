/* Stand-in header: forwards to the one-rank shim (test infrastructure only). */
#ifndef GBMV_SHIM_MPI_H
#define GBMV_SHIM_MPI_H
#include <math.h>
#include "shim_core.h"
#endif
