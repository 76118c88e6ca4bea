// sbp_petsc.cpp -- the PETSc-facing adapter of libsbpgpu (include/sbp_petsc.h):
// the RHS callback PETSc's TS calls once per stage, and drop-ins for the
// reference's ts_rk4 / ts_rk45 that run the whole integration on the device.
// Built into libsbpgpu_petsc.so by build.py's build_petsc_adapter() where
// PETSc's headers are found; the repository's tests build it against a minimal
// stand-in of the same PETSc calls.
#include "sbp_petsc.h"

#if defined(PETSC_USE_COMPLEX) || !defined(PETSC_USE_REAL_DOUBLE)
#error "the adapter passes PETSc's arrays to the library as double: it needs a real, double-precision PETSc"
#endif

namespace {

// The vector holds one state of the context's problem.
PetscErrorCode check_size(sbp_ctx* c, Vec v, const char* which) {
  PetscInt n = 0;
  PetscCall(VecGetLocalSize(v, &n));
  PetscCheck((long long)n == sbp_size(c), PETSC_COMM_SELF, PETSC_ERR_ARG_SIZ,
             "%s has %lld local entries, the context's state %lld", which, (long long)n, sbp_size(c));
  return PETSC_SUCCESS;
}

}  // namespace

extern "C" PetscErrorCode sbp_petsc_rhs(TS ts, PetscReal t, Vec src, Vec dst, void* ctx) {
  (void)ts;
  sbp_ctx* c = static_cast<sbp_ctx*>(ctx);
  PetscCheck(c != nullptr, PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "sbp_petsc_rhs: the context must be an sbp_ctx*");
  PetscCall(check_size(c, src, "src"));
  PetscCall(check_size(c, dst, "dst"));
  const PetscScalar* s = nullptr;
  PetscScalar* d = nullptr;
  PetscCall(VecGetArrayRead(src, &s));
  PetscCall(VecGetArrayWrite(dst, &d));
  const int rc = sbp_rhs(c, (double)t, s, d, SBP_HOST);
  PetscCall(VecRestoreArrayWrite(dst, &d));
  PetscCall(VecRestoreArrayRead(src, &s));
  PetscCheck(rc == SBP_OK, PETSC_COMM_SELF, PETSC_ERR_LIB, "sbp_rhs: %s", sbp_last_error(c));
  return PETSC_SUCCESS;
}

extern "C" PetscErrorCode sbp_petsc_ts_rk4(sbp_ctx* c, PetscReal t_end, PetscReal dt, Vec v) {
  PetscCheck(c != nullptr, PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "sbp_petsc_ts_rk4: null context");
  PetscCall(check_size(c, v, "v"));
  PetscScalar* a = nullptr;
  PetscCall(VecGetArray(v, &a));
  const int rc = sbp_ts_rk4(c, (double)t_end, (double)dt, a, SBP_HOST);
  PetscCall(VecRestoreArray(v, &a));
  PetscCheck(rc == SBP_OK, PETSC_COMM_SELF, PETSC_ERR_LIB, "sbp_ts_rk4: %s", sbp_last_error(c));
  return PETSC_SUCCESS;
}

extern "C" PetscErrorCode sbp_petsc_ts_rk45(sbp_ctx* c, PetscReal t_end, PetscReal dt, Vec v) {
  PetscCheck(c != nullptr, PETSC_COMM_SELF, PETSC_ERR_ARG_NULL, "sbp_petsc_ts_rk45: null context");
  PetscCall(check_size(c, v, "v"));
  PetscScalar* a = nullptr;
  PetscCall(VecGetArray(v, &a));
  const int rc = sbp_ts_rk45(c, (double)t_end, (double)dt, a, SBP_HOST);
  PetscCall(VecRestoreArray(v, &a));
  PetscCheck(rc != SBP_ERR_DIVERGED, PETSC_COMM_SELF, PETSC_ERR_NOT_CONVERGED, "sbp_ts_rk45: %s",
             sbp_last_error(c));
  PetscCheck(rc == SBP_OK, PETSC_COMM_SELF, PETSC_ERR_LIB, "sbp_ts_rk45: %s", sbp_last_error(c));
  return PETSC_SUCCESS;
}
