/*
 * A minimal stand-in for the PETSc calls the adapter (include/sbp_petsc.h)
 * makes -- test infrastructure: PETSc is not installed where the tests run.
 * Vectors are host arrays that track whether their array is checked out, so
 * a test can see every VecGetArray* matched by its VecRestoreArray*. Error
 * codes are distinct small numbers with PETSc's names; shim_last_error()
 * keeps the message of the last failed check.
 */
#ifndef SBP_TEST_PETSC_SHIM_H
#define SBP_TEST_PETSC_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int PetscErrorCode;
typedef double PetscReal;
typedef double PetscScalar;
typedef int PetscInt;
typedef struct ShimVec* Vec;
typedef struct ShimTS* TS;

#define PETSC_USE_REAL_DOUBLE 1
#define PETSC_SUCCESS 0
#define PETSC_COMM_SELF 0
#define PETSC_ERR_ARG_SIZ 60
#define PETSC_ERR_ARG_NULL 85
#define PETSC_ERR_LIB 76
#define PETSC_ERR_NOT_CONVERGED 91
#define PETSC_ERR_ARG_WRONGSTATE 73

PetscErrorCode shim_error(PetscErrorCode code, const char* fmt, ...);
const char* shim_last_error(void);

#define PetscCall(call)                  \
  do {                                   \
    PetscErrorCode shim_e_ = (call);     \
    if (shim_e_) return shim_e_;         \
  } while (0)
#define PetscCheck(cond, comm, code, ...)                  \
  do {                                                     \
    if (!(cond)) return shim_error((code), __VA_ARGS__);   \
  } while (0)

PetscErrorCode VecGetLocalSize(Vec v, PetscInt* n);
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar** a);
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar** a);
PetscErrorCode VecGetArrayWrite(Vec v, PetscScalar** a);
PetscErrorCode VecRestoreArrayWrite(Vec v, PetscScalar** a);
PetscErrorCode VecGetArray(Vec v, PetscScalar** a);
PetscErrorCode VecRestoreArray(Vec v, PetscScalar** a);

/* test helpers */
Vec shim_vec_create(PetscInt n);
void shim_vec_destroy(Vec v);
PetscScalar* shim_vec_data(Vec v);   /* the array, without checking it out */
int shim_vec_checked_out(Vec v);     /* arrays currently checked out */

#ifdef __cplusplus
}
#endif

#endif
