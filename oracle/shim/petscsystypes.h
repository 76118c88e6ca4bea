/*
 * Stand-in for PETSc's petscsystypes.h, so that the reference's header-only
 * SBP operators and RHS kernels compile without PETSc. Test infrastructure
 * only: it is used to build oracle/_ref, the checker, never the product.
 *
 * Only what the hot-path headers touch is provided: the scalar/int typedefs,
 * PETSC_PI, PetscSqrtReal and a one-rank MPIU_Allreduce (a copy), which is
 * what H_central::get_norm_1D (code/include/sbpops/H_central.h:99) does on
 * a single rank.
 */
#pragma once
#include <cmath>
typedef long long PetscInt;
typedef double PetscScalar;
typedef double PetscReal;
#define PETSC_COMM_WORLD 0
#define MPIU_REAL 0
#define MPIU_SUM 0
#define MPIU_Allreduce(in, out, n, type, op, comm) (*(out) = *(in))
#define PetscSqrtReal(x) std::sqrt(x)
#define PETSC_PI 3.14159265358979323846264
