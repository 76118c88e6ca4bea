// sbp_demo.cpp -- the reference's demo drivers through the C ABI of libsbpgpu.
//
// Mirrors the flow of the reference's main programs: set up a grid, fill the
// initial data, time the time stepper, compare with the exact solution and
// print "Elapsed time: ... seconds" and "The l2-error is: ..., and the maximum
// error is ..." as they do (code/demo/wave_hom/wave_eq_hom_sim.cpp:53-200,
// code/demo/advection/advection_1D_sim.cpp). The PETSc DMDA, TS and MPI set-up
// of those programs becomes one sbp_create and one sbp_ts_rk4 call; the arrays
// keep the DMDA's AoS layout.
//
//   sbp_demo wave_hom Nx Ny Tend CFL [order]          standing mode (n, m) = (3, 4),
//                                                     free-surface SAT, dt = CFL / min(hix, hiy)
//   sbp_demo advection_1d N Tend CFL [order] [a]      Gaussian exp(-(x - a t)^2 / 0.1^2) on
//                                                     [-1, 1], inflow SAT, dt = CFL / hi
//                                                     (the reference program fixes a = 1.5)
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "sbpgpu.h"

namespace {

const double kPi = 3.14159265358979323846;

// Standing mode of wave_eq_hom_sim.cpp:211-233, components (u, v, p).
void wave_hom_exact(std::vector<double>& v, long long nx, long long ny, double h0, double h1, double t) {
  const int n = 3, m = 4;
  const double w = std::sqrt((double)(n * n + m * m));
  for (long long j = 0; j < ny; j++) {
    const double y = -1.0 + j * h1;
    for (long long i = 0; i < nx; i++) {
      const double x = -1.0 + i * h0;
      double* q = &v[3 * (i + nx * j)];
      q[0] = -n * std::cos(n * kPi * x) * std::sin(m * kPi * y) * std::sin(kPi * w * t) / w;
      q[1] = -m * std::sin(n * kPi * x) * std::cos(m * kPi * y) * std::sin(kPi * w * t) / w;
      q[2] = std::sin(kPi * n * x) * std::sin(kPi * m * y) * std::cos(kPi * w * t);
    }
  }
}

// Advected Gaussian of advection_1D_sim.cpp:171-188.
void adv1d_exact(std::vector<double>& v, long long n, double h, double a, double t) {
  for (long long i = 0; i < n; i++) {
    const double x = -1.0 + i * h - a * t;
    v[i] = std::exp(-x * x / (0.1 * 0.1));
  }
}

int usage(const char* prog) {
  std::fprintf(stderr,
               "usage: %s wave_hom Nx Ny Tend CFL [order]\n"
               "       %s advection_1d N Tend CFL [order] [a]\n",
               prog, prog);
  return 1;
}

int fail(sbp_ctx* ctx, const char* what, int rc) {
  std::fprintf(stderr, "%s failed (%d): %s\n", what, rc, ctx ? sbp_last_error(ctx) : sbp_last_error(nullptr));
  return 2;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) return usage(argv[0]);
  const bool wave = std::strcmp(argv[1], "wave_hom") == 0;
  const bool adv = std::strcmp(argv[1], "advection_1d") == 0;
  if ((!wave && !adv) || (wave && (argc < 6 || argc > 7)) || (adv && (argc < 5 || argc > 7))) return usage(argv[0]);
  sbp_desc d;
  std::memset(&d, 0, sizeof(d));
  d.bc = SBP_BC_REFERENCE;
  d.precision = SBP_FP64;
  d.xl[0] = d.xl[1] = -1.0;
  d.xr[0] = d.xr[1] = 1.0;
  double tend, cfl, a = 1.5;
  if (wave) {
    d.problem = SBP_WAVE_HOM_2D;
    d.nx = std::atoll(argv[2]);
    d.ny = std::atoll(argv[3]);
    tend = std::atof(argv[4]);
    cfl = std::atof(argv[5]);
    d.order = argc > 6 ? std::atoi(argv[6]) : 4;
  } else {
    d.problem = SBP_ADVECTION_1D;
    d.nx = std::atoll(argv[2]);
    d.ny = 1;
    tend = std::atof(argv[3]);
    cfl = std::atof(argv[4]);
    d.order = argc > 5 ? std::atoi(argv[5]) : 4;
    if (argc > 6) a = std::atof(argv[6]);
    d.a = a;
  }
  if (d.nx <= 0 || d.ny <= 0 || !(tend > 0) || !(cfl > 0)) return usage(argv[0]);
  sbp_ctx* ctx = nullptr;
  int rc = sbp_create(&d, &ctx);
  if (rc) return fail(nullptr, "sbp_create", rc);
  const long long dofs = sbp_dofs(ctx), n = d.nx * d.ny * dofs;
  const double h0 = 2.0 / (d.nx - 1), h1 = wave ? 2.0 / (d.ny - 1) : 1.0;
  // time step of the reference programs: CFL / min(hi) (2D), CFL / hi (1D)
  const double dt = wave ? cfl / std::fmin(1.0 / h0, 1.0 / h1) : cfl * h0;
  std::vector<double> v(n), exact(n);
  if (wave)
    wave_hom_exact(v, d.nx, d.ny, h0, h1, 0.0);
  else
    adv1d_exact(v, d.nx, h0, a, 0.0);
  const auto t0 = std::chrono::steady_clock::now();
  rc = sbp_ts_rk4(ctx, tend, dt, v.data(), SBP_HOST);
  const auto t1 = std::chrono::steady_clock::now();
  if (rc) return fail(ctx, "sbp_ts_rk4", rc);
  std::printf("Elapsed time: %f seconds\n", std::chrono::duration<double>(t1 - t0).count());
  if (wave)
    wave_hom_exact(exact, d.nx, d.ny, h0, h1, tend);
  else
    adv1d_exact(exact, d.nx, h0, a, tend);
  double l2 = 0, mx = 0;
  if ((rc = sbp_set_state(ctx, v.data(), SBP_HOST)) || (rc = sbp_error_norms(ctx, exact.data(), SBP_HOST, &l2, &mx)))
    return fail(ctx, "sbp_error_norms", rc);
  std::printf("The l2-error is: %g, and the maximum error is %g\n", l2, mx);
  sbp_destroy(ctx);
  return 0;
}
