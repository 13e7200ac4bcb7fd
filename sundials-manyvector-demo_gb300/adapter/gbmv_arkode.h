/* ARKODE-signature callbacks over the gbmv C ABI: the bodies a SUNDIALS 6 build of the
 * reference's drivers registers in place of its own right-hand sides, Jacobian, block linear
 * solver and rank-local MRI inner stepper, over MPIManyVectors whose six components are device
 * arrays (fluid rho, mx, my, mz, et, then the species-fastest chemistry).
 *
 * This translation unit needs the SUNDIALS headers (sundials/, nvector/, sunmatrix/,
 * arkode/) and links against libgbmv.so; it is not part of libgbmv.so, which depends on no
 * SUNDIALS.  Every callback returns the ARKODE convention: 0 success, > 0 recoverable, < 0
 * unrecoverable.
 */
#ifndef GBMV_ARKODE_H
#define GBMV_ARKODE_H

#include <arkode/arkode_mristep.h>
#include <sundials/sundials_linearsolver.h>
#include <sundials/sundials_matrix.h>
#include <sundials/sundials_nvector.h>

#include "gbmv.h"

#ifdef __cplusplus
extern "C" {
#endif

/* user_data of the callbacks (the device counterpart of the reference's EulerData plus its
 * cvklu_data): handles, units, the WENO arithmetic, the stream, the inner DIRK's options. */
typedef struct {
  gbmv_hydro hydro;
  gbmv_chem chem;          /* NULL for pure hydrodynamics */
  double energy_units;     /* EulerData::EnergyUnits */
  double time_units;       /* EulerData::TimeUnits */
  double cfl;              /* EulerData::cfl (stability) */
  int precision;           /* GBMV_FP64 / GBMV_MIXED / GBMV_MIXED_FAST for the flux divergence */
  void* stream;            /* cudaStream_t of every call */
  gbmv_dirk_opts fast_opts; /* the inner (fast) DIRK of the MRI stepper */
} gbmv_arkode_data;

/* content of the MRI inner stepper and user_data of ffast (the reference's
 * RankLocalStepperContent, src/multirate_chem_hydro_main.cpp:92-97) */
typedef struct {
  gbmv_arkode_data* data;
  MRIStepInnerStepper stepper;  /* source of the forcing data */
  int disable_forcing;          /* 1 while ffast is evaluated without the MRI forcing */
} gbmv_inner_content;

/* ARKRhsFn, replaces fEuler (src/utilities.cpp:17-253) */
int gbmv_ark_feuler(realtype t, N_Vector w, N_Vector wdot, void* user_data);
/* ARKRhsFn, replaces fexpl / fslow (src/imex_chem_hydro_main.cpp:910-1000,
 * src/multirate_chem_hydro_main.cpp:996-1083) */
int gbmv_ark_fexpl(realtype t, N_Vector w, N_Vector wdot, void* user_data);
/* ARKRhsFn, replaces fimpl (src/imex_chem_hydro_main.cpp:811-848): fluid 0, chemistry
 * TimeUnits x source */
int gbmv_ark_fimpl(realtype t, N_Vector w, N_Vector wdot, void* user_data);
/* ARKRhsFn, replaces ffast (src/multirate_chem_hydro_main.cpp:897-946), the MRI forcing
 * included; user_data is a gbmv_inner_content */
int gbmv_ark_ffast(realtype t, N_Vector w, N_Vector wdot, void* user_data);
/* ARKLsJacFn, replaces Jimpl / Jfast (src/imex_chem_hydro_main.cpp:850-908,
 * src/multirate_chem_hydro_main.cpp:954-994): J a SUNMatrix_MagmaDenseBlock of 10 x 10 blocks */
int gbmv_ark_jac(realtype t, N_Vector w, N_Vector fw, SUNMatrix J, void* user_data,
                 N_Vector tmp1, N_Vector tmp2, N_Vector tmp3);
/* ARKPostProcessFn, replaces PostprocessStep (src/imex_chem_hydro_main.cpp:1002-1051) */
int gbmv_ark_postprocess(realtype t, N_Vector w, void* user_data);
/* ARKStabilityFn, replaces stability (src/utilities.cpp:483-528) */
int gbmv_ark_stability(N_Vector w, realtype t, realtype* dt_stab, void* user_data);

/* SUNLinearSolver of type DIRECT on subvector `subvec` of the ManyVectors it is given (the
 * chemistry, 5), factoring the block matrix ARKLS formed (A = I - gamma J) in place:
 * replaces SUNLinSol_RankLocalLS / SUNLinSol_BDMPIMV over MAGMA's batched getrf / getrs
 * (src/multirate_chem_hydro_main.cpp:1312-1411, src/imex_chem_hydro_main.cpp:1075-1194).
 * Returns NULL on failure. */
SUNLinearSolver gbmv_SUNLinSol_Block(N_Vector x, sunindextype subvec, gbmv_arkode_data* data,
                                     SUNContext ctx);

/* MRIStepInnerStepper hooks of the rank-local inner stepper, content a gbmv_inner_content:
 * evolve replaces RankLocalStepper_Evolve (the whole fast integration to tout in one
 * persistent launch of the batched DIRK, src/multirate_chem_hydro_main.cpp:1114-1160), fullrhs
 * RankLocalStepper_FullRhs (ffast without forcing, :1165-1200) and reset
 * RankLocalStepper_Reset (:1203-1224: nothing to reset, the DIRK keeps no history). */
int gbmv_inner_evolve(MRIStepInnerStepper stepper, realtype t0, realtype tout, N_Vector y);
int gbmv_inner_fullrhs(MRIStepInnerStepper stepper, realtype t, N_Vector y, N_Vector f,
                       int mode);
int gbmv_inner_reset(MRIStepInnerStepper stepper, realtype tR, N_Vector yR);

#ifdef __cplusplus
}
#endif
#endif
