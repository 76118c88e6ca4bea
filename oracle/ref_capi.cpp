/*
 * C API over the reference's own hot-path headers. TEST INFRASTRUCTURE ONLY:
 * this file is compiled (by oracle/Makefile, from the headers where they lie
 * in the reference checkout) into oracle/_ref/libsbpref.so, which pins the
 * C restatement in oracle/sbp_oracle.c and generates tests/golden/ fixtures.
 * Nothing in the product links it.
 *
 * One translation unit per (problem, order): op_defs.h selects the operator
 * by the SBP_OPERATOR_ORDER macro (code/include/sbpops/op_defs.h:7-30), and
 * wave_eq_rhs.h / wave_eq_hom_rhs.h both define free_surface_bc_* templates,
 * so they cannot share a unit. REF_PROBLEM picks the demo header; the order
 * suffix keeps the symbols of the nine units apart in one library.
 *
 * Every array argument is the reference's own AoS format: element
 * (j, i, comp) at dofs*(i + nx*j) + comp (code/include/grids/layout.h:124-127).
 */
#include <array>
#include <vector>
#include "sbpops/op_defs.h"

#define CAT3(a, b, c) a##b##c
#define XCAT3(a, b, c) CAT3(a, b, c)
#define SYM(name) XCAT3(name, _o, SBP_OPERATOR_ORDER)

#if REF_PROBLEM == 1
#include "wave_hom/wave_eq_hom_rhs.h"

/* The matrix-free apply wave_eq_hom_serial (code/demo/wave_hom/wave_eq_hom_rhs.h:365). */
extern "C" void SYM(ref_wave_hom_apply)(long long nx, long long ny, double hix, double hiy,
                                        double xl0, double xl1, double t,
                                        const double* src, double* dst) {
  const FirstDerivativeOp D1;
  grid::partitioned_layout_2d L(grid::extents_2d(nx, ny, 3), 0, nx, ny);
  grid::grid_function_2d<PetscScalar> q(const_cast<double*>(src), L), F(dst, L);
  wave_eq_hom_serial(F, q, D1, std::array<double, 2>{hix, hiy}, std::array<double, 2>{xl0, xl1}, t);
}

/* The free-surface SAT wave_eq_hom_free_surface_bc_serial (wave_eq_hom_rhs.h:443). */
extern "C" void SYM(ref_wave_hom_bc)(long long nx, long long ny, double hix, double hiy,
                                     const double* src, double* dst) {
  const InverseNormOp HI;
  grid::partitioned_layout_2d L(grid::extents_2d(nx, ny, 3), 0, nx, ny);
  grid::grid_function_2d<PetscScalar> q(const_cast<double*>(src), L), F(dst, L);
  wave_eq_hom_free_surface_bc_serial(F, q, HI, std::array<double, 2>{hix, hiy});
}
#elif REF_PROBLEM == 2
/* wave_eq_rhs.h defines rho_inv/forcing_u/forcing_v as non-inline functions;
 * rename them per order so the three order units link into one library. */
#define rho_inv SYM(rho_inv)
#define forcing_u SYM(forcing_u)
#define forcing_v SYM(forcing_v)
#include "wave/wave_eq_rhs.h"

/* wave_eq_serial: variable density 1/(2+xy) and manufactured forcing (code/demo/wave/wave_eq_rhs.h:389). */
extern "C" void SYM(ref_wave_apply)(long long nx, long long ny, double hix, double hiy,
                                    double xl0, double xl1, double t,
                                    const double* src, double* dst) {
  const FirstDerivativeOp D1;
  grid::partitioned_layout_2d L(grid::extents_2d(nx, ny, 3), 0, nx, ny);
  grid::grid_function_2d<PetscScalar> q(const_cast<double*>(src), L), F(dst, L);
  wave_eq_serial(F, q, D1, std::array<double, 2>{hix, hiy}, std::array<double, 2>{xl0, xl1}, t);
}

extern "C" void SYM(ref_wave_bc)(long long nx, long long ny, double hix, double hiy,
                                 const double* src, double* dst) {
  const InverseNormOp HI;
  grid::partitioned_layout_2d L(grid::extents_2d(nx, ny, 3), 0, nx, ny);
  grid::grid_function_2d<PetscScalar> q(const_cast<double*>(src), L), F(dst, L);
  wave_eq_free_surface_bc_serial(F, q, HI, std::array<double, 2>{hix, hiy});
}
#elif REF_PROBLEM == 3
#include "advection/advection_rhs.h"

/* advection_serial + advection_bc_serial, 1D (code/demo/advection/advection_rhs.h:83,133). */
extern "C" void SYM(ref_adv1d_apply)(long long n, double hi, double a, const double* src, double* dst) {
  const FirstDerivativeOp D1;
  auto vel = [a](const PetscInt) { return a; };
  grid::partitioned_layout_1d L(grid::extents_1d(n, 1), 0, n);
  grid::grid_function_1d<PetscScalar> s(const_cast<double*>(src), L), d(dst, L);
  advection_serial(d, s, D1, hi, vel);
}

extern "C" void SYM(ref_adv1d_bc)(long long n, double hi, double a, const double* src, double* dst) {
  const InverseNormOp HI;
  auto vel = [a](const PetscInt) { return a; };
  grid::partitioned_layout_1d L(grid::extents_1d(n, 1), 0, n);
  grid::grid_function_1d<PetscScalar> s(const_cast<double*>(src), L), d(dst, L);
  advection_bc_serial(d, s, HI, hi, vel);
}

/* advection_serial + advection_bc_serial, 2D (advection_rhs.h:440,531). */
extern "C" void SYM(ref_adv2d_apply)(long long nx, long long ny, double hix, double hiy,
                                     double a, double b, const double* src, double* dst) {
  const FirstDerivativeOp D1;
  std::function<double(PetscInt, PetscInt)> va = [a](PetscInt, PetscInt) { return a; };
  std::function<double(PetscInt, PetscInt)> vb = [b](PetscInt, PetscInt) { return b; };
  grid::partitioned_layout_2d L(grid::extents_2d(nx, ny, 1), 0, nx, ny);
  grid::grid_function_2d<PetscScalar> s(const_cast<double*>(src), L), d(dst, L);
  advection_serial(d, s, D1, std::array<double, 2>{hix, hiy}, va, vb);
}

extern "C" void SYM(ref_adv2d_bc)(long long nx, long long ny, double hix, double hiy,
                                  double a, double b, const double* src, double* dst) {
  const InverseNormOp HI;
  std::function<double(PetscInt, PetscInt)> va = [a](PetscInt, PetscInt) { return a; };
  std::function<double(PetscInt, PetscInt)> vb = [b](PetscInt, PetscInt) { return b; };
  grid::partitioned_layout_2d L(grid::extents_2d(nx, ny, 1), 0, nx, ny);
  grid::grid_function_2d<PetscScalar> s(const_cast<double*>(src), L), d(dst, L);
  advection_bc_serial(d, s, HI, std::array<double, 2>{hix, hiy}, va, vb);
}
/* The same with a velocity at every point, the reference's callable a(i)
 * (advection_1D_sim.cpp:19): a[i]. */
extern "C" void SYM(ref_adv1d_apply_var)(long long n, double hi, const double* a, const double* src, double* dst) {
  const FirstDerivativeOp D1;
  auto vel = [a](const PetscInt i) { return a[i]; };
  grid::partitioned_layout_1d L(grid::extents_1d(n, 1), 0, n);
  grid::grid_function_1d<PetscScalar> s(const_cast<double*>(src), L), d(dst, L);
  advection_serial(d, s, D1, hi, vel);
}

extern "C" void SYM(ref_adv1d_bc_var)(long long n, double hi, const double* a, const double* src, double* dst) {
  const InverseNormOp HI;
  auto vel = [a](const PetscInt i) { return a[i]; };
  grid::partitioned_layout_1d L(grid::extents_1d(n, 1), 0, n);
  grid::grid_function_1d<PetscScalar> s(const_cast<double*>(src), L), d(dst, L);
  advection_bc_serial(d, s, HI, hi, vel);
}

/* 2D with velocity fields a(i,j) = a[i + nx*j], b(i,j) = b[i + nx*j]. */
extern "C" void SYM(ref_adv2d_apply_var)(long long nx, long long ny, double hix, double hiy, const double* a,
                                         const double* b, const double* src, double* dst) {
  const FirstDerivativeOp D1;
  std::function<double(PetscInt, PetscInt)> va = [a, nx](PetscInt i, PetscInt j) { return a[i + nx * j]; };
  std::function<double(PetscInt, PetscInt)> vb = [b, nx](PetscInt i, PetscInt j) { return b[i + nx * j]; };
  grid::partitioned_layout_2d L(grid::extents_2d(nx, ny, 1), 0, nx, ny);
  grid::grid_function_2d<PetscScalar> s(const_cast<double*>(src), L), d(dst, L);
  advection_serial(d, s, D1, std::array<double, 2>{hix, hiy}, va, vb);
}

extern "C" void SYM(ref_adv2d_bc_var)(long long nx, long long ny, double hix, double hiy, const double* a,
                                      const double* b, const double* src, double* dst) {
  const InverseNormOp HI;
  std::function<double(PetscInt, PetscInt)> va = [a, nx](PetscInt i, PetscInt j) { return a[i + nx * j]; };
  std::function<double(PetscInt, PetscInt)> vb = [b, nx](PetscInt i, PetscInt j) { return b[i + nx * j]; };
  grid::partitioned_layout_2d L(grid::extents_2d(nx, ny, 1), 0, nx, ny);
  grid::grid_function_2d<PetscScalar> s(const_cast<double*>(src), L), d(dst, L);
  advection_bc_serial(d, s, HI, std::array<double, 2>{hix, hiy}, va, vb);
}
#elif REF_PROBLEM == 4
#include "reflection/reflection_rhs.h"

/* reflection_serial + reflection_bc_serial (code/demo/reflection/reflection_rhs.h:98,129). */
extern "C" void SYM(ref_refl_apply)(long long n, double hi, const double* src, double* dst) {
  const FirstDerivativeOp D1;
  grid::partitioned_layout_1d L(grid::extents_1d(n, 2), 0, n);
  grid::grid_function_1d<PetscScalar> s(const_cast<double*>(src), L), d(dst, L);
  reflection_serial(d, s, D1, hi);
}

extern "C" void SYM(ref_refl_bc)(long long n, const double* src, double* dst) {
  grid::partitioned_layout_1d L(grid::extents_1d(n, 2), 0, n);
  grid::grid_function_1d<PetscScalar> s(const_cast<double*>(src), L), d(dst, L);
  reflection_bc_serial(d, s);
}

/* H_central::get_norm_1D on one rank (code/include/sbpops/H_central.h:70-103). */
extern "C" double SYM(ref_hnorm1d)(long long n, long long dofs, double h, const double* v) {
  const NormOp H;
  std::vector<const double*> rows(n);
  for (long long i = 0; i < n; i++) rows[i] = v + i * dofs;
  return H.get_norm_1D(const_cast<const PetscScalar* const*>(rows.data()), h, n, 0, n, dofs);
}
#else
#error "REF_PROBLEM must be 1..4"
#endif
