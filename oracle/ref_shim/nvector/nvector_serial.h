/* Stand-in header: forwards to the one-rank shim (test infrastructure only). */
#ifndef GBMV_SHIM_NVECTOR_NVECTOR_SERIAL_H
#define GBMV_SHIM_NVECTOR_NVECTOR_SERIAL_H
#include <math.h>
#include "../shim_core.h"
#endif
