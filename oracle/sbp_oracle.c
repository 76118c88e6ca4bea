/*
 * sbp_oracle.c -- CPU restatement of the reference's matrix-free SBP-SAT
 * right-hand sides, RK4 and norms (VidarStiernstrom/HPC-reading-course).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the "port" CPU
 * baseline of bench.py. The product never links or calls this file.
 *
 * Arithmetic follows the reference operation by operation (tap order,
 * hi * sum after the sum, left-to-right products), so that built with
 * -ffp-contract=off it reproduces the reference's headers bit for bit; the
 * CPU tests pin it against fixtures generated from those headers.
 */
#include "sbp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* SBP first-derivative operators: interior stencil and left closure block
 * (code/include/sbpops/D1_central.h:243-273). */
static const double D1_INT_2[3] = {-1. / 2, 0, 1. / 2};
static const double D1_CLS_2[1][2] = {{-1., 1}};
static const double D1_INT_4[5] = {1. / 12, -2. / 3, 0., 2. / 3, -1. / 12};
static const double D1_CLS_4[4][6] = {{-24. / 17, 59. / 34, -4. / 17, -3. / 34, 0, 0},
                                      {-1. / 2, 0, 1. / 2, 0, 0, 0},
                                      {4. / 43, -59. / 86, 0, 59. / 86, -4. / 43, 0},
                                      {3. / 98, 0, -59. / 98, 0, 32. / 49, -4. / 49}};
static const double D1_INT_6[7] = {-1. / 60, 3. / 20, -3. / 4, 0, 3. / 4, -3. / 20, 1. / 60};
static const double D1_CLS_6[6][9] = {
    {-21600. / 13649, 104009. / 54596, 30443. / 81894, -33311. / 27298, 16863. / 27298, -15025. / 163788, 0, 0, 0},
    {-104009. / 240260, 0, -311. / 72078, 20229. / 24026, -24337. / 48052, 36661. / 360390, 0, 0, 0},
    {-30443. / 162660, 311. / 32532, 0, -11155. / 16266, 41287. / 32532, -21999. / 54220, 0, 0, 0},
    {33311. / 107180, -20229. / 21436, 485. / 1398, 0, 4147. / 21436, 25427. / 321540, 72. / 5359, 0, 0},
    {-16863. / 78770, 24337. / 31508, -41287. / 47262, -4147. / 15754, 0, 342523. / 472620, -1296. / 7877, 144. / 7877, 0},
    {15025. / 525612, -36661. / 262806, 21999. / 87602, -25427. / 262806, -342523. / 525612, 0, 32400. / 43801, -6480. / 43801, 720. / 43801}};

/* Inverse quadrature weights of the closures (code/include/sbpops/HI_central.h:128-147). */
static const double HI_2[1] = {2.};
static const double HI_4[4] = {48. / 17, 48. / 59, 48. / 43, 48. / 49};
static const double HI_6[6] = {43200. / 13649, 8640. / 12013, 4320. / 2711, 4320. / 5359, 8640. / 7877, 43200. / 43801};

/* Quadrature weights of the closures (code/include/sbpops/H_central.h:193-212). */
static const double H_2[1] = {1. / 2};
static const double H_4[4] = {17. / 48, 59. / 48, 43. / 48, 49. / 48};
static const double H_6[6] = {13649. / 43200, 12013. / 8640, 2711. / 4320, 5359. / 4320, 7877. / 8640, 43801. / 43200};

#define ORC_PI 3.14159265358979323846264

/* rho_inv (code/demo/wave/wave_eq_rhs.h:42-46): x = xl + i/hi, 1/(2 + x y). */
static inline double mms_rho_inv(const orc_problem* p, long long i, long long j) {
  const double x = p->xl0 + (double)i / p->hix;
  const double y = p->xl1 + (double)j / p->hiy;
  return 1. / (2 + x * y);
}

/* forcing_u (wave_eq_rhs.h:51-55). */
static inline double mms_forcing_u(const orc_problem* p, long long i, long long j, double t) {
  const double x = p->xl0 + (double)i / p->hix;
  const double y = p->xl1 + (double)j / p->hiy;
  return -(3 * ORC_PI * cos(5 * ORC_PI * t) * cos(3 * ORC_PI * x) * sin(4 * ORC_PI * y) * (x * y + 1)) / (x * y + 2);
}

/* forcing_v (wave_eq_rhs.h:60-64). */
static inline double mms_forcing_v(const orc_problem* p, long long i, long long j, double t) {
  const double x = p->xl0 + (double)i / p->hix;
  const double y = p->xl1 + (double)j / p->hiy;
  return -(4 * ORC_PI * cos(5 * ORC_PI * t) * cos(4 * ORC_PI * y) * sin(3 * ORC_PI * x) * (x * y + 1)) / (x * y + 2);
}

#define ORD 2
#include "sbp_oracle_body.inc"
#undef ORD
#define ORD 4
#include "sbp_oracle_body.inc"
#undef ORD
#define ORD 6
#include "sbp_oracle_body.inc"
#undef ORD

int orc_dofs(int problem) {
  switch (problem) {
    case ORC_WAVE_HOM_2D:
    case ORC_WAVE_MMS_2D:
    case ORC_WAVE_VAR_2D:
    case ORC_WAVE_2BLOCK_2D: return 3;
    case ORC_WAVE_3D: return 4;
    case ORC_ADVECTION_1D:
    case ORC_ADVECTION_2D: return 1;
    case ORC_REFLECTION_1D: return 2;
    default: return -1;
  }
}

long long orc_min_points(int order) {
  switch (order) {
    case 2: return 3;
    case 4: return 8;
    case 6: return 12;
    default: return -1;
  }
}

static int is_2d(int problem) {
  return problem == ORC_WAVE_HOM_2D || problem == ORC_WAVE_MMS_2D || problem == ORC_WAVE_VAR_2D ||
         problem == ORC_ADVECTION_2D || problem == ORC_WAVE_2BLOCK_2D;
}

/* Scalars of a state of problem p. */
static long long nscalars(const orc_problem* p) {
  const long long pts = p->nx * (is_2d(p->problem) || p->problem == ORC_WAVE_3D ? p->ny : 1) *
                        (p->problem == ORC_WAVE_3D ? p->nz : 1);
  return pts * orc_dofs(p->problem);
}

static int check(const orc_problem* p) {
  if (!p || orc_dofs(p->problem) < 0) return -1;
  const long long m = orc_min_points(p->order);
  if (m < 0) return -2;
  if (p->nx < m) return -3;
  if (is_2d(p->problem) && p->ny < m) return -3;
  if (p->problem == ORC_WAVE_3D && (p->ny < m || p->nz < m)) return -3;
  if ((p->problem == ORC_WAVE_VAR_2D || p->problem == ORC_WAVE_2BLOCK_2D) && (!p->rho || !p->K)) return -4;
  if (p->problem == ORC_WAVE_2BLOCK_2D && (p->ny % 2 || p->ny / 2 < m)) return -3;
  return 0;
}

#define DISPATCH(call_prefix, ...)                                        \
  switch (p->order) {                                                     \
    case 2: call_prefix##_o2(__VA_ARGS__); break;                          \
    case 4: call_prefix##_o4(__VA_ARGS__); break;                          \
    default: call_prefix##_o6(__VA_ARGS__); break;                         \
  }

int orc_apply(const orc_problem* p, double t, const double* src, double* dst) {
  const int rc = check(p);
  if (rc) return rc;
  switch (p->problem) {
    case ORC_WAVE_HOM_2D: DISPATCH(wave_hom_apply, p, src, dst); break;
    case ORC_WAVE_MMS_2D: DISPATCH(wave_mms_apply, p, t, src, dst); break;
    case ORC_WAVE_VAR_2D: DISPATCH(wave_var_apply, p, src, dst); break;
    case ORC_WAVE_2BLOCK_2D: DISPATCH(wave_2block_apply, p, src, dst); break;
    case ORC_WAVE_3D: DISPATCH(wave3d_apply, p, src, dst); break;
    case ORC_ADVECTION_1D: DISPATCH(adv1d_apply, p, src, dst); break;
    case ORC_ADVECTION_2D: DISPATCH(adv2d_apply, p, src, dst); break;
    case ORC_REFLECTION_1D: DISPATCH(refl_apply, p, src, dst); break;
  }
  return 0;
}

int orc_bc(const orc_problem* p, const double* src, double* dst) {
  const int rc = check(p);
  if (rc) return rc;
  switch (p->problem) {
    case ORC_WAVE_HOM_2D:
      if (p->bc == ORC_BC_CHARACTERISTIC) {
        DISPATCH(wave_hom_char_bc, p, src, dst);
      } else {
        DISPATCH(wave_free_surface_bc, p, src, dst);
      }
      break;
    case ORC_WAVE_MMS_2D: DISPATCH(wave_free_surface_bc, p, src, dst); break;
    case ORC_WAVE_VAR_2D: DISPATCH(wave_var_bc, p, src, dst); break;
    case ORC_WAVE_2BLOCK_2D: DISPATCH(wave_2block_bc, p, src, dst); break;
    case ORC_WAVE_3D: DISPATCH(wave3d_bc, p, src, dst); break;
    case ORC_ADVECTION_1D: DISPATCH(adv1d_bc, p, src, dst); break;
    case ORC_ADVECTION_2D: DISPATCH(adv2d_bc, p, src, dst); break;
    case ORC_REFLECTION_1D: /* proj_dirichlet_bc_{l,r} (reflection_rhs.h:108-120) */
      dst[0] = 0.0;
      dst[2 * (p->nx - 1)] = 0.0;
      break;
  }
  return 0;
}

int orc_rhs(const orc_problem* p, double t, const double* src, double* dst) {
  int rc = orc_apply(p, t, src, dst);
  if (rc) return rc;
  return orc_bc(p, src, dst);
}

void orc_rk45_default_opts(orc_rk45_opts* o) {
  o->atol = 1e-4;
  o->rtol = 1e-4;
  o->safety = 0.9;
  o->reject_safety = 0.5;
  o->clip_lo = 0.1;
  o->clip_hi = 10.0;
  o->dt_min = 1e-20;
  o->dt_max = 1e50;
  o->max_steps = 10000000;
  o->max_reject = 10;
}

/* Fehlberg's 4(5) pair. */
static const double RKF_C[6] = {0.0, 1.0 / 4, 3.0 / 8, 12.0 / 13, 1.0, 1.0 / 2};
static const double RKF_A[6][5] = {{0, 0, 0, 0, 0},
                                   {1.0 / 4, 0, 0, 0, 0},
                                   {3.0 / 32, 9.0 / 32, 0, 0, 0},
                                   {1932.0 / 2197, -7200.0 / 2197, 7296.0 / 2197, 0, 0},
                                   {439.0 / 216, -8.0, 3680.0 / 513, -845.0 / 4104, 0},
                                   {-8.0 / 27, 2.0, -3544.0 / 2565, 1859.0 / 4104, -11.0 / 40}};
static const double RKF_B5[6] = {16.0 / 135, 0.0, 6656.0 / 12825, 28561.0 / 56430, -9.0 / 50, 2.0 / 55};
static const double RKF_B4[6] = {25.0 / 216, 0.0, 1408.0 / 2565, 2197.0 / 4104, -1.0 / 5, 0.0};

/* Landing rule on t_end for a candidate step h0 from t; sets *fin on the last step. */
static double rk45_land(double t, double t_end, double h0, int* fin) {
  const double hmax = t_end - t;
  double h = h0;
  *fin = 0;
  if (h0 >= hmax) {
    *fin = 1;
    return hmax;
  }
  if (2.0 * h0 > hmax) h = 0.5 * hmax;
  if (1.01 * h0 > hmax) {
    h = hmax;
    *fin = 1;
  }
  return h;
}

int orc_rk45(const orc_problem* p, double t0, double t_end, double dt0, const orc_rk45_opts* opts, double* v,
             orc_rk45_stats* st) {
  int rc = check(p);
  if (rc) return rc;
  orc_rk45_opts o;
  if (opts) o = *opts; else orc_rk45_default_opts(&o);
  const long long n = nscalars(p);
  double* k[6];
  double* w = (double*)malloc(sizeof(double) * n);
  double* u5 = (double*)malloc(sizeof(double) * n);
  int ok = w && u5;
  for (int s = 0; s < 6; s++) {
    k[s] = (double*)malloc(sizeof(double) * n);
    ok = ok && k[s];
  }
  if (!ok) {
    free(w); free(u5);
    for (int s = 0; s < 6; s++) free(k[s]);
    return -5;
  }
  double t = t0, wlte = 0.0;
  long long acc = 0, rej = 0;
  int last_ok = 1, in_row = 0, fin = 0, status = 0, done = !(t_end > t0);
  double h = rk45_land(t0, t_end, fmin(dt0, o.dt_max), &fin);
  while (!done) {
    for (int s = 0; s < 6; s++) {
      const double* in = v;
      if (s > 0) {
#pragma omp parallel for schedule(static) if (n > 65536)
        for (long long i = 0; i < n; i++) {
          double a = RKF_A[s][0] * k[0][i];
          for (int j = 1; j < s; j++) a = fma(RKF_A[s][j], k[j][i], a);
          w[i] = fma(h, a, v[i]);
        }
        in = w;
      }
      orc_rhs(p, t + RKF_C[s] * h, in, k[s]);
    }
    double sum = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : sum) if (n > 65536)
    for (long long i = 0; i < n; i++) {
      double s5 = RKF_B5[0] * k[0][i], s4 = RKF_B4[0] * k[0][i];
      for (int j = 1; j < 6; j++) {
        s5 = fma(RKF_B5[j], k[j][i], s5);
        s4 = fma(RKF_B4[j], k[j][i], s4);
      }
      const double a5 = fma(h, s5, v[i]), a4 = fma(h, s4, v[i]);
      u5[i] = a5;
      const double tol = o.atol + o.rtol * fmax(fabs(a5), fabs(a4));
      if (tol != 0.0) { /* a zero tolerance contributes 0 */
        const double e = (a5 - a4) / tol;
        sum += e * e;
      }
    }
    wlte = sqrt(sum / (double)n);
    if (!(wlte <= 1e300)) {
      rej++;
      status = 2;
      break;
    }
    double safety = o.safety;
    int accept = 1;
    if (wlte > 1.0) {
      if (!last_ok) safety *= o.reject_safety;
      accept = h < (1.0 + 1.4901161193847656e-08) * o.dt_min;
    }
    double hfac = wlte > 0.0 ? safety * pow(wlte, -0.2) : o.clip_hi;
    hfac = fmin(fmax(hfac, o.clip_lo), o.clip_hi);
    double hn = fmin(fmax(h * hfac, o.dt_min), o.dt_max);
    last_ok = accept;
    if (accept) {
      memcpy(v, u5, sizeof(double) * n);
      acc++;
      in_row = 0;
      if (fin) {
        t = t_end;
        h = hn;
        break;
      }
      t = t + h;
    } else {
      rej++;
      in_row++;
    }
    h = rk45_land(t, t_end, hn, &fin);
    if (in_row >= o.max_reject) {
      status = 3;
      break;
    }
    if (acc + rej >= o.max_steps) {
      status = 1;
      break;
    }
  }
  if (st) {
    st->accepted = acc;
    st->rejected = rej;
    st->t = t;
    st->dt_next = h;
    st->wlte = wlte;
    st->status = status;
  }
  free(w); free(u5);
  for (int s = 0; s < 6; s++) free(k[s]);
  return 0;
}

long long orc_rk4_nsteps(double t_end, double* dt_inout) {
  const double dt = *dt_inout;
  const long long n = llround(t_end / dt);
  if (n > 0 && fabs((double)n * dt - t_end) > 1e-14) *dt_inout = t_end / (double)n;
  return n;
}

/* RK4_custom's stage arithmetic (code/include/time_stepping/time_stepping.h:127-142):
 * tmp = v + dt/2 k1, tmp = v + dt/2 k2, tmp = v + dt k3 (apply_WAXPY :232-252),
 * v += dt/6 (k1 + 2 (k2 + k3) + k4) (rk4_util :254-278). */
int orc_rk4(const orc_problem* p, double t0, double dt, long long nsteps, double* v) {
  int rc = check(p);
  if (rc) return rc;
  const long long n = nscalars(p);
  double* k1 = (double*)malloc(sizeof(double) * n);
  double* k2 = (double*)malloc(sizeof(double) * n);
  double* k3 = (double*)malloc(sizeof(double) * n);
  double* k4 = (double*)malloc(sizeof(double) * n);
  double* tmp = (double*)malloc(sizeof(double) * n);
  if (!k1 || !k2 || !k3 || !k4 || !tmp) {
    free(k1); free(k2); free(k3); free(k4); free(tmp);
    return -5;
  }
  const double h2 = 0.5 * dt, h6 = dt / 6;
  double t = t0;
  for (long long s = 0; s < nsteps; s++) {
    orc_rhs(p, t, v, k1);
#pragma omp parallel for schedule(static) if (n > 65536)
    for (long long i = 0; i < n; i++) tmp[i] = v[i] + h2 * k1[i];
    orc_rhs(p, t + h2, tmp, k2);
#pragma omp parallel for schedule(static) if (n > 65536)
    for (long long i = 0; i < n; i++) tmp[i] = v[i] + h2 * k2[i];
    orc_rhs(p, t + h2, tmp, k3);
#pragma omp parallel for schedule(static) if (n > 65536)
    for (long long i = 0; i < n; i++) tmp[i] = v[i] + dt * k3[i];
    orc_rhs(p, t + dt, tmp, k4);
#pragma omp parallel for schedule(static) if (n > 65536)
    for (long long i = 0; i < n; i++) v[i] += h6 * (k1[i] + 2 * (k2[i] + k3[i]) + k4[i]);
    t = t + dt;
  }
  free(k1); free(k2); free(k3); free(k4); free(tmp);
  return 0;
}

double orc_hnorm1d_reference(const double* v, long long n, long long dofs, double h, int order) {
  switch (order) {
    case 2: return hnorm1d_reference_o2(v, n, dofs, h);
    case 4: return hnorm1d_reference_o4(v, n, dofs, h);
    case 6: return hnorm1d_reference_o6(v, n, dofs, h);
    default: return -1;
  }
}

double orc_hnorm_2block(const double* v, long long nx, long long ny, long long dofs, double hx, double hy,
                        int order) {
  switch (order) {
    case 2: return hnorm_2block_o2(v, nx, ny, dofs, hx, hy);
    case 4: return hnorm_2block_o4(v, nx, ny, dofs, hx, hy);
    case 6: return hnorm_2block_o6(v, nx, ny, dofs, hx, hy);
    default: return -1;
  }
}

double orc_hnorm(const double* v, long long nx, long long ny, long long dofs, double hx, double hy, int order) {
  switch (order) {
    case 2: return hnorm_o2(v, nx, ny, dofs, hx, hy);
    case 4: return hnorm_o4(v, nx, ny, dofs, hx, hy);
    case 6: return hnorm_o6(v, nx, ny, dofs, hx, hy);
    default: return -1;
  }
}

double orc_hnorm3d(const double* v, long long nx, long long ny, long long nz, long long dofs, double hx, double hy,
                   double hz, int order) {
  switch (order) {
    case 2: return hnorm3d_o2(v, nx, ny, nz, dofs, hx, hy, hz);
    case 4: return hnorm3d_o4(v, nx, ny, nz, dofs, hx, hy, hz);
    case 6: return hnorm3d_o6(v, nx, ny, nz, dofs, hx, hy, hz);
    default: return -1;
  }
}

/* error_l2: sqrt(prod h) * ||v1 - v2||_2 over every component (vec_util.h:47-57). */
double orc_error_l2(const double* v1, const double* v2, long long n, double hprod) {
  double s = 0;
  for (long long i = 0; i < n; i++) {
    const double e = fabs(v2[i] - v1[i]);
    s += e * e;
  }
  return sqrt(hprod) * sqrt(s);
}

/* error_max: ||v1 - v2||_inf (vec_util.h:59-61). */
double orc_error_max(const double* v1, const double* v2, long long n) {
  double m = 0;
  for (long long i = 0; i < n; i++) {
    const double e = fabs(v2[i] - v1[i]);
    if (e > m) m = e;
  }
  return m;
}

void orc_init_adv1d(double* v, long long n, double xl, double h, double a, double t) {
  const double rstar = 0.1;
  for (long long i = 0; i < n; i++) {
    const double x = xl + i * h - a * t;
    v[i] = exp(-x * x / (rstar * rstar));
  }
}

void orc_init_adv2d(double* v, long long nx, long long ny, double xl0, double xl1,
                    double hx, double hy, double a, double b, double t) {
  const double rstar = 0.1;
  for (long long j = 0; j < ny; j++) {
    const double y = xl1 + j * hy - b * t;
    for (long long i = 0; i < nx; i++) {
      const double x = xl0 + i * hx - a * t;
      v[i + nx * j] = exp(-(x * x + y * y) / (rstar * rstar));
    }
  }
}

void orc_init_wave_mms(double* v, long long nx, long long ny, double xl0, double xl1,
                       double hx, double hy, double t) {
  const int n = 3, m = 4;
  for (long long j = 0; j < ny; j++) {
    const double y = xl1 + j * hy;
    for (long long i = 0; i < nx; i++) {
      const double x = xl0 + i * hx;
      double* q = v + 3 * (i + nx * j);
      q[0] = -n * cos(n * ORC_PI * x) * sin(m * ORC_PI * y) * sin(ORC_PI * sqrt(n * n + m * m) * t) / sqrt(n * n + m * m);
      q[1] = -m * sin(n * ORC_PI * x) * cos(m * ORC_PI * y) * sin(ORC_PI * sqrt(n * n + m * m) * t) / sqrt(n * n + m * m);
      q[2] = sin(ORC_PI * n * x) * sin(ORC_PI * m * y) * cos(ORC_PI * sqrt(n * n + m * m) * t);
    }
  }
}

static double theta1(double x, double t) {
  const double rstar = 0.1;
  return exp(-(x - t) * (x - t) / (rstar * rstar));
}

void orc_init_reflection(double* v, long long n, double xl, double h, double t, double W) {
  for (long long i = 0; i < n; i++) {
    const double x = xl + i * h;
    if (t == 0.0) {
      v[2 * i + 0] = -theta1(x, 0) - theta1(x, 0);
      v[2 * i + 1] = -theta1(x, 0) + theta1(x, 0);
    } else {
      v[2 * i + 0] = theta1(x, W - t) + theta1(x, -W + t);
      v[2 * i + 1] = theta1(x, W - t) - theta1(x, -W + t);
    }
  }
}

void orc_init_wave_pulse(double* v, long long nx, long long ny, double xl0, double xl1,
                         double hx, double hy, double x0, double y0, double w, double amp) {
  for (long long j = 0; j < ny; j++) {
    const double y = xl1 + j * hy - y0;
    for (long long i = 0; i < nx; i++) {
      const double x = xl0 + i * hx - x0;
      double* q = v + 3 * (i + nx * j);
      q[0] = 0.0;
      q[1] = 0.0;
      q[2] = amp * exp(-(x * x + y * y) / (w * w));
    }
  }
}

void orc_init_wave3d_mode(double* v, long long nx, long long ny, long long nz, double xl0, double xl1, double xl2,
                          double hx, double hy, double hz, int a, int b, int c, double t) {
  const double w = ORC_PI * sqrt((double)(a * a + b * b + c * c));
  const double ka = a * ORC_PI, kb = b * ORC_PI, kc = c * ORC_PI;
  for (long long k = 0; k < nz; k++) {
    const double z = xl2 + k * hz;
    for (long long j = 0; j < ny; j++) {
      const double y = xl1 + j * hy;
      for (long long i = 0; i < nx; i++) {
        const double x = xl0 + i * hx;
        double* q = v + 4 * (i + nx * (j + ny * k));
        const double sx = sin(ka * x), sy = sin(kb * y), sz = sin(kc * z);
        q[0] = -(ka / w) * sin(w * t) * cos(ka * x) * sy * sz;
        q[1] = -(kb / w) * sin(w * t) * sx * cos(kb * y) * sz;
        q[2] = -(kc / w) * sin(w * t) * sx * sy * cos(kc * z);
        q[3] = cos(w * t) * sx * sy * sz;
      }
    }
  }
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
