/* The stand-in's vectors and error record (test infrastructure; see petscts.h). */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>

#include "petscts.h"

struct ShimVec {
  PetscInt n;
  PetscScalar* a;
  int out;
};

static char g_msg[512];

PetscErrorCode shim_error(PetscErrorCode code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof(g_msg), fmt, ap);
  va_end(ap);
  return code;
}

const char* shim_last_error(void) { return g_msg; }

Vec shim_vec_create(PetscInt n) {
  Vec v = (Vec)calloc(1, sizeof(struct ShimVec));
  v->n = n;
  v->a = (PetscScalar*)calloc((size_t)(n > 0 ? n : 1), sizeof(PetscScalar));
  return v;
}

void shim_vec_destroy(Vec v) {
  if (!v) return;
  free(v->a);
  free(v);
}

PetscScalar* shim_vec_data(Vec v) { return v->a; }
int shim_vec_checked_out(Vec v) { return v->out; }

PetscErrorCode VecGetLocalSize(Vec v, PetscInt* n) {
  if (!v || !n) return shim_error(PETSC_ERR_ARG_NULL, "VecGetLocalSize: null argument");
  *n = v->n;
  return PETSC_SUCCESS;
}

static PetscErrorCode get(Vec v, PetscScalar** a) {
  if (!v || !a) return shim_error(PETSC_ERR_ARG_NULL, "VecGetArray*: null argument");
  if (v->out) return shim_error(PETSC_ERR_ARG_WRONGSTATE, "VecGetArray*: array already checked out");
  v->out = 1;
  *a = v->a;
  return PETSC_SUCCESS;
}

static PetscErrorCode put(Vec v, PetscScalar** a) {
  if (!v || !a) return shim_error(PETSC_ERR_ARG_NULL, "VecRestoreArray*: null argument");
  if (!v->out || *a != v->a) return shim_error(PETSC_ERR_ARG_WRONGSTATE, "VecRestoreArray*: not checked out");
  v->out = 0;
  *a = NULL;
  return PETSC_SUCCESS;
}

PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar** a) { return get(v, (PetscScalar**)a); }
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar** a) { return put(v, (PetscScalar**)a); }
PetscErrorCode VecGetArrayWrite(Vec v, PetscScalar** a) { return get(v, a); }
PetscErrorCode VecRestoreArrayWrite(Vec v, PetscScalar** a) { return put(v, a); }
PetscErrorCode VecGetArray(Vec v, PetscScalar** a) { return get(v, a); }
PetscErrorCode VecRestoreArray(Vec v, PetscScalar** a) { return put(v, a); }
