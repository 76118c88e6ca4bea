/*
 * sbp_oracle.h -- CPU restatement of the reference's SBP-SAT hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA path
 * and the timed CPU baseline ("port") in bench.py. The product never links,
 * loads or calls it.
 *
 * Arrays use the reference's AoS format: element (j, i, comp) of a grid with
 * nx points in x and `dofs` components lives at dofs*(i + nx*j) + comp
 * (code/include/grids/layout.h:124-127, 1D: layout.h:65-68).
 *
 * Parity is pinned: tests/golden/ holds outputs of the reference's own
 * headers (built as oracle/_ref by oracle/Makefile) and the CPU tests check
 * this restatement against them bit for bit where no libm call is involved.
 */
#ifndef SBP_ORACLE_H
#define SBP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum orc_problem_kind {
  ORC_WAVE_HOM_2D = 1,  /* rho = K = 1, code/demo/wave_hom/wave_eq_hom_rhs.h */
  ORC_WAVE_MMS_2D = 2,  /* rho^-1 = 1/(2+xy) + forcing, code/demo/wave/wave_eq_rhs.h */
  ORC_ADVECTION_1D = 3, /* code/demo/advection/advection_rhs.h:12-140 */
  ORC_ADVECTION_2D = 4, /* code/demo/advection/advection_rhs.h:155-558 */
  ORC_REFLECTION_1D = 5,/* code/demo/reflection/reflection_rhs.h */
  ORC_WAVE_VAR_2D = 6,  /* rho(x,y), K(x,y) fields; no reference counterpart */
  ORC_WAVE_2BLOCK_2D = 7,/* two ORC_WAVE_VAR_2D blocks (rows [0,ny/2) and [ny/2,ny)) sharing the
                            interface line y = (xl1+xr1)/2, coupled by an interface SAT */
  ORC_WAVE_3D = 8        /* 3D acoustic wave (u, v, w, p), rho = K = 1; no reference counterpart
                            (3D is a TODO at code/include/partitioned_rhs/rhs.h:400-402) */
};

enum orc_bc_kind {
  ORC_BC_REFERENCE = 0,      /* the problem's own BC in the reference */
  ORC_BC_CHARACTERISTIC = 1  /* ORC_WAVE_VAR_2D, ORC_WAVE_2BLOCK_2D, ORC_WAVE_3D and ORC_WAVE_HOM_2D (rho = K = 1): non-reflecting SAT */
};

typedef struct {
  int problem;        /* orc_problem_kind */
  int order;          /* 2, 4 or 6 */
  int bc;             /* orc_bc_kind */
  long long nx, ny;   /* points (ny = 1 in 1D) */
  double hix, hiy;    /* inverse spacings (N-1)/(xr-xl) */
  double xl0, xl1;    /* lower-left corner */
  double a, b;        /* advection velocities */
  const double* rho;  /* ORC_WAVE_VAR_2D: nx*ny density, row-major (j,i) */
  const double* K;    /* ORC_WAVE_VAR_2D: nx*ny bulk modulus */
  long long nz;       /* ORC_WAVE_3D: points in z (element (k, j, i, comp) at dofs*(i + nx*(j + ny*k)) + comp) */
  double hiz, xl2;    /* ORC_WAVE_3D: inverse z spacing, lower z bound */
  const double* va;   /* advection: velocity a at every point (1D: nx; 2D: nx*ny, row-major (j,i)), or NULL for a */
  const double* vb;   /* 2D advection: velocity b at every point, or NULL for b */
} orc_problem;

/* ORC_WAVE_2BLOCK_2D: each block has ny/2 points in y over half the domain,
 * hiy = (ny/2 - 1) / ((xr1 - xl1)/2); the last row of the lower block and the
 * first row of the upper block are the same physical line. rho and K cover
 * all nx*ny points (each block's own values on the interface line). */

/* Number of components per grid point of a problem kind. */
int orc_dofs(int problem);

/* Minimum points per direction for an order: max(closure width, 2*closure size). */
long long orc_min_points(int order);

/* The matrix-free apply (interior stencils + closures, no boundary terms). */
int orc_apply(const orc_problem* p, double t, const double* src, double* dst);
/* The boundary terms added to dst (SAT penalties, or projection). */
int orc_bc(const orc_problem* p, const double* src, double* dst);
/* The full RHS callback body: orc_apply then orc_bc. */
int orc_rhs(const orc_problem* p, double t, const double* src, double* dst);

/* Classical RK4, nsteps of size dt from t0, in place on v
 * (code/include/time_stepping/time_stepping.h:127-142). */
int orc_rk4(const orc_problem* p, double t0, double dt, long long nsteps, double* v);

/* Adaptive Runge-Kutta-Fehlberg 4(5) with the basic step-size controller, from
 * t0 to t_end in place on v. Restates what the reference's ts_rk45
 * (code/src/time_stepping/ts_rk.cpp:41-52) asks of PETSc: TSRK5F (Fehlberg's
 * published pair, E. Fehlberg, NASA TR R-315, 1969, advanced with the 5th-order
 * weights) under TSADAPTBASIC with TS_EXACTFINALTIME_MATCHSTEP and default
 * options. PETSc is an unpinned dependency absent from the reference tree; the
 * controller is restated from its documented behaviour:
 *   wlte = sqrt(mean_i (|u5_i - u4_i| / (atol + rtol max(|u5_i|, |u4_i|)))^2),
 *   an entry with a zero tolerance contributing 0
 *   accept iff wlte <= 1 (or h < (1 + sqrt(eps)) dt_min)
 *   safety' = safety * reject_safety if this and the previous attempt failed
 *   h' = clamp(h * clamp(safety' wlte^(-1/5), clip_lo, clip_hi), dt_min, dt_max)
 *   with hmax = t_end - t: h' >= hmax -> hmax (last step); otherwise
 *   2 h' > hmax -> hmax / 2, then 1.01 h' > hmax -> hmax (last step).
 * The first attempt is dt0 under the same landing rule. Stops when the last
 * step is accepted (t = t_end), after max_reject rejections in a row (status
 * 3), after max_steps attempts (status 1) or on a non-finite wlte (status 2).
 * Stage inputs w = u + h * (a_s1 k1 + ...), sums left to right with fma. */
typedef struct {
  double atol, rtol, safety, reject_safety, clip_lo, clip_hi, dt_min, dt_max;
  long long max_steps;
  int max_reject;
} orc_rk45_opts;
typedef struct {
  long long accepted, rejected;
  double t, dt_next, wlte;
  int status;
} orc_rk45_stats;
void orc_rk45_default_opts(orc_rk45_opts* o);
int orc_rk45(const orc_problem* p, double t0, double t_end, double dt0, const orc_rk45_opts* o, double* v,
             orc_rk45_stats* st);

/* Step count rule of the reference's RK4: round(t_end/dt) steps, and dt is
 * replaced by t_end/steps when they do not match (time_stepping.h:104-109). */
long long orc_rk4_nsteps(double t_end, double* dt_inout);

/* H-norm exactly as H_central::get_norm_1D computes it on one rank
 * (code/include/sbpops/H_central.h:70-103): left-closure weights only. */
double orc_hnorm1d_reference(const double* v, long long n, long long dofs, double h, int order);
/* H-norm with both closures, 1D or 2D (tensor product); nx*ny points. */
double orc_hnorm(const double* v, long long nx, long long ny, long long dofs,
                 double hx, double hy, int order);

/* H-norm of a 3D state (tensor product of the three 1D quadratures). */
double orc_hnorm3d(const double* v, long long nx, long long ny, long long nz, long long dofs, double hx, double hy,
                   double hz, int order);

/* H-norm of a two-block state (ny/2 rows per block, each block's quadrature). */
double orc_hnorm_2block(const double* v, long long nx, long long ny, long long dofs, double hx, double hy,
                        int order);

/* Discrete L2 error sqrt(prod h) * ||v1 - v2||_2 and max error
 * (code/include/util/vec_util.h:47-61). n = total scalars. */
double orc_error_l2(const double* v1, const double* v2, long long n, double hprod);
double orc_error_max(const double* v1, const double* v2, long long n);

/* Initial / exact data of the reference demos, AoS. */
/* 1D advected Gaussian exp(-(x-a t)^2/0.1^2) (advection_1D_sim.cpp:171-188). */
void orc_init_adv1d(double* v, long long n, double xl, double h, double a, double t);
/* 2D advected Gaussian (advection_2D_sim.cpp:188-209). */
void orc_init_adv2d(double* v, long long nx, long long ny, double xl0, double xl1,
                    double hx, double hy, double a, double b, double t);
/* Standing mode n=3, m=4 (wave_eq_hom_sim.cpp:211-233), components u, v, p. */
void orc_init_wave_mms(double* v, long long nx, long long ny, double xl0, double xl1,
                       double hx, double hy, double t);
/* Reflection pulses (reflection_sim.cpp:177-225): t = 0 gives the initial
 * condition, otherwise the exact solution with width W. */
void orc_init_reflection(double* v, long long n, double xl, double h, double t, double W);
/* Standing mode of ORC_WAVE_3D with p = 0 on the faces of [-1,1]^3 (a, b, c integers):
 * p = cos(w t) sin(a pi x) sin(b pi y) sin(c pi z), u = -(a pi / w) sin(w t) cos(a pi x) sin(b pi y)
 * sin(c pi z) (v, w alike), w = pi sqrt(a^2 + b^2 + c^2); components (u, v, w, p). */
void orc_init_wave3d_mode(double* v, long long nx, long long ny, long long nz, double xl0, double xl1, double xl2,
                          double hx, double hy, double hz, int a, int b, int c, double t);
/* Gaussian pressure pulse p0 = amp*exp(-((x-x0)^2+(y-y0)^2)/w^2), u = v = 0. */
void orc_init_wave_pulse(double* v, long long nx, long long ny, double xl0, double xl1,
                         double hx, double hy, double x0, double y0, double w, double amp);

/* Threads used by the OpenMP loops (0 = leave the runtime default). */
void orc_set_threads(int n);
int orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
