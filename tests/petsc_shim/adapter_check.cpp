// Drives the PETSc adapter (hpc-reading-course_gb300/petsc/sbp_petsc.cpp) through
// the stand-in's vectors -- test infrastructure.
//   adapter_check cpu  argument and error paths that need no device
//   adapter_check gpu  also: sbp_petsc_rhs / sbp_petsc_ts_rk4 give the bits of
//                      sbp_rhs / sbp_ts_rk4 on a 2D wave context; a failing library
//                      call comes back as PETSC_ERR_LIB with the arrays restored
// Prints one line per check; exit status 0 when all pass.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "sbp_petsc.h"

static int g_fail = 0;
#define CHECK(cond, what)                                              \
  do {                                                                 \
    const bool ok_ = (cond);                                           \
    std::printf("%s %s\n", ok_ ? "ok  " : "FAIL", what);               \
    if (!ok_) g_fail = 1;                                              \
  } while (0)

int main(int argc, char** argv) {
  const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
  Vec a = shim_vec_create(12), b = shim_vec_create(12);
  CHECK(sbp_petsc_rhs(nullptr, 0.0, a, b, nullptr) == PETSC_ERR_ARG_NULL, "rhs: null context");
  CHECK(sbp_petsc_ts_rk4(nullptr, 1.0, 0.1, a) == PETSC_ERR_ARG_NULL, "ts_rk4: null context");
  CHECK(sbp_petsc_ts_rk45(nullptr, 1.0, 0.1, a) == PETSC_ERR_ARG_NULL, "ts_rk45: null context");
  CHECK(!shim_vec_checked_out(a) && !shim_vec_checked_out(b), "no array left checked out");
  shim_vec_destroy(a);
  shim_vec_destroy(b);
  if (!gpu) return g_fail;

  const int nx = 40, ny = 30, order = 4;
  sbp_desc d;
  std::memset(&d, 0, sizeof(d));
  d.problem = SBP_WAVE_HOM_2D;
  d.order = order;
  d.bc = SBP_BC_REFERENCE;
  d.precision = SBP_FP64;
  d.nx = nx;
  d.ny = ny;
  d.xl[0] = d.xl[1] = -1.0;
  d.xr[0] = d.xr[1] = 1.0;
  sbp_ctx* c = nullptr;
  CHECK(sbp_create(&d, &c) == SBP_OK, "sbp_create");
  if (!c) return 1;
  const long long n = sbp_size(c);
  CHECK(n == 3LL * nx * ny, "sbp_size");
  Vec src = shim_vec_create((PetscInt)n), dst = shim_vec_create((PetscInt)n), bad = shim_vec_create((PetscInt)n - 1);
  for (long long k = 0; k < n; k++) shim_vec_data(src)[k] = std::sin(0.37 * (double)k) + 0.1 * std::cos(1.3 * (double)k);
  std::vector<double> ref(n);
  CHECK(sbp_petsc_rhs(nullptr, 0.25, src, dst, c) == PETSC_SUCCESS, "rhs through the adapter");
  CHECK(sbp_rhs(c, 0.25, shim_vec_data(src), ref.data(), SBP_HOST) == SBP_OK, "rhs direct");
  CHECK(std::memcmp(ref.data(), shim_vec_data(dst), n * sizeof(double)) == 0, "rhs: the same bits");
  CHECK(sbp_petsc_rhs(nullptr, 0.0, src, bad, c) == PETSC_ERR_ARG_SIZ, "rhs: wrong vector size");
  const double h = 2.0 / (nx - 1), dt = 0.2 * h;
  std::vector<double> v(shim_vec_data(src), shim_vec_data(src) + n);
  CHECK(sbp_petsc_ts_rk4(c, 10 * dt, dt, src) == PETSC_SUCCESS, "ts_rk4 through the adapter");
  CHECK(sbp_ts_rk4(c, 10 * dt, dt, v.data(), SBP_HOST) == SBP_OK, "ts_rk4 direct");
  CHECK(std::memcmp(v.data(), shim_vec_data(src), n * sizeof(double)) == 0, "ts_rk4: the same bits");
  CHECK(sbp_petsc_ts_rk4(c, -1.0, dt, src) == PETSC_ERR_LIB, "ts_rk4: a failing call is PETSC_ERR_LIB");
  CHECK(std::strstr(shim_last_error(), "sbp_ts_rk4") != nullptr, "the error names the call");
  CHECK(!shim_vec_checked_out(src) && !shim_vec_checked_out(dst) && !shim_vec_checked_out(bad),
        "no array left checked out");
  shim_vec_destroy(src);
  shim_vec_destroy(dst);
  shim_vec_destroy(bad);
  sbp_destroy(c);
  return g_fail;
}
