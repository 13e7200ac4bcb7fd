/* Stand-in header: the ARKStep and generic SUNDIALS calls the reference's main programs make
 * (src/imex_chem_hydro_main.cpp), declared so that the file compiles on one rank; none of them
 * runs when only its callbacks (fexpl, PostprocessStep) are called.  Test infrastructure only:
 * oracle/ref_glue.cpp includes that file to reach its callbacks. */
#ifndef GBMV_SHIM_ARKODE_ARKODE_ARKSTEP_H
#define GBMV_SHIM_ARKODE_ARKODE_ARKSTEP_H
#include <math.h>
#include "../shim_core.h"
#include "../shim_glue.h"
#endif
