/*
 * sbp_petsc.h -- the PETSc-facing adapter of libsbpgpu (libsbpgpu_petsc.so,
 * built from hpc-reading-course_gb300/petsc/sbp_petsc.cpp where PETSc's
 * headers are found). It makes the library a literal drop-in for the
 * reference's driver calls on a single-rank DMDA vector (real FP64, AoS,
 * dofs*(i + nx*j) + comp: code/include/grids/layout.h:124-127):
 *
 *   TSSetRHSFunction(ts, NULL, sbp_petsc_rhs, ctx)  for  TSSetRHSFunction(ts, NULL, rhs, &appctx)
 *                                                    (code/src/time_stepping/ts_rk.cpp:21)
 *   sbp_petsc_ts_rk4(ctx, t_end, dt, v)              for  ts_rk4(da, t_end, dt, v, rhs, &appctx)
 *                                                    (ts_rk.cpp:54-65)
 *   sbp_petsc_ts_rk45(ctx, t_end, dt, v)             for  ts_rk45(da, t_end, dt, v, rhs, &appctx)
 *                                                    (ts_rk.cpp:41-52)
 *
 * ctx is the sbp_ctx* of sbp_create. Errors come back as PETSc error codes:
 * a null context PETSC_ERR_ARG_NULL, a vector whose local size is not
 * sbp_size(ctx) PETSC_ERR_ARG_SIZ, a failed library call PETSC_ERR_LIB (its
 * sbp_last_error message in the PETSc error), an adaptive integration that
 * stopped early PETSC_ERR_NOT_CONVERGED. Every array taken from a vector is
 * given back before the function returns.
 */
#ifndef SBP_PETSC_H
#define SBP_PETSC_H

#include <petscts.h>

#include "sbpgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

PetscErrorCode sbp_petsc_rhs(TS ts, PetscReal t, Vec src, Vec dst, void* ctx);
PetscErrorCode sbp_petsc_ts_rk4(sbp_ctx* ctx, PetscReal t_end, PetscReal dt, Vec v);
PetscErrorCode sbp_petsc_ts_rk45(sbp_ctx* ctx, PetscReal t_end, PetscReal dt, Vec v);

#ifdef __cplusplus
}
#endif

#endif
