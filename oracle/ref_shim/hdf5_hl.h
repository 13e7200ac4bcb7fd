/* Stand-in header: forwards to the one-rank shim (test infrastructure only). */
#ifndef GBMV_SHIM_HDF5_HL_H
#define GBMV_SHIM_HDF5_HL_H
#include <math.h>
#include "shim_core.h"
#endif
