/*
 * sbpgpu.h -- C ABI of the GB300 (sm_103a) implementation of the matrix-free
 * SBP-SAT hot path of VidarStiernstrom/HPC-reading-course: the right-hand
 * side of first-order hyperbolic systems with summation-by-parts first
 * derivatives of order 2, 4 or 6, SAT boundary terms, and the classical RK4
 * time stepper that calls it.
 *
 * Library: hpc-reading-course_gb300/lib/libsbpgpu.so. Plain C types only.
 * Every function returns an int status (SBP_OK = 0, negative on error) and
 * never throws; sbp_last_error() gives the message of the last failure on a
 * context. A context is bound to one CUDA stream and one device; calls on one
 * context must not run concurrently (as the reference's callbacks, which run
 * one per MPI rank). Device arrays passed in are read and written on that
 * stream: a caller that produces or consumes them on another stream orders
 * the two first (an event, or a synchronize).
 *
 * Array format at the boundary is the reference's: FP64, array-of-structs,
 * element (j, i, comp) at dofs*(i + nx*j) + comp (code/include/grids/layout.h:124-127;
 * 1D: layout.h:65-68), the layout a single-rank PETSc DMDA vector has.
 * `where` says whether such an array is in host memory (SBP_HOST) or device
 * memory (SBP_DEVICE). Inside the library the state is device-resident
 * structure-of-arrays with padded rows.
 */
#ifndef SBPGPU_H
#define SBPGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define SBP_OK 0
#define SBP_ERR_INVALID (-1)     /* bad argument (size, order, pointer, problem) */
#define SBP_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define SBP_ERR_DEVICE (-3)      /* a kernel reported an error (e.g. a bounded wait gave up) */
#define SBP_ERR_UNSUPPORTED (-4) /* combination not provided (e.g. FP32 manufactured-solution problem) */
#define SBP_ERR_TOO_LARGE (-5)   /* grid exceeds the static scratch of sbp_wave_rhs_noalloc */
#define SBP_ERR_DIVERGED (-6)    /* the adaptive integrator stopped before t_end (see sbp_rk45_stats) */

/* Problems: the reference demos plus the variable-coefficient wave system. */
typedef enum {
  SBP_WAVE_HOM_2D = 1,   /* code/demo/wave_hom: (u,v,p), rho = K = 1 */
  SBP_WAVE_MMS_2D = 2,   /* code/demo/wave: rho^-1 = 1/(2+xy), manufactured forcing */
  SBP_ADVECTION_1D = 3,  /* code/demo/advection, u_t + a u_x = 0 */
  SBP_ADVECTION_2D = 4,  /* code/demo/advection, u_t + a u_x + b u_y = 0 */
  SBP_REFLECTION_1D = 5, /* code/demo/reflection, [u;v]_t = [v_x;u_x] */
  SBP_WAVE_VAR_2D = 6,   /* (u,v,p) with rho(x,y), K(x,y) fields; no reference counterpart */
  SBP_WAVE_2BLOCK_2D = 7,/* two SBP_WAVE_VAR_2D blocks, rows [0,ny/2) and [ny/2,ny), sharing the
                            line y = (xl[1]+xr[1])/2 (stored in both blocks), coupled by an
                            energy-conserving interface SAT; no reference counterpart */
  SBP_WAVE_3D = 8        /* (u,v,w,p), rho = K = 1, on nx x ny x nz points: the wave_hom system with a
                            third direction (the reference leaves 3D as a TODO,
                            code/include/partitioned_rhs/rhs.h:400-402); free-surface or
                            characteristic SAT on the six faces. Arrays: element (k, j, i, comp)
                            at 4*(i + nx*(j + ny*k)) + comp */
} sbp_problem;

typedef enum {
  SBP_BC_REFERENCE = 0,      /* the demo's own boundary treatment: free-surface SAT
                                (wave), inflow SAT (advection), projection (reflection) */
  SBP_BC_CHARACTERISTIC = 1  /* wave problems: non-reflecting SAT on p + Z u_n */
} sbp_bc;

typedef enum { SBP_FP64 = 0, SBP_FP32 = 1 } sbp_precision;
typedef enum { SBP_HOST = 0, SBP_DEVICE = 1 } sbp_where;

typedef struct sbp_ctx sbp_ctx;

/* Problem description; the fields play the role of the reference's AppCtx
 * (code/demo/wave_hom/wave_eq_hom_sim.cpp:36-45) plus the compile-time order
 * of op_defs.h (code/include/sbpops/op_defs.h:7-30). */
typedef struct {
  int problem;        /* sbp_problem */
  int order;          /* 2, 4 or 6 */
  int bc;             /* sbp_bc */
  int precision;      /* sbp_precision: SBP_FP32 keeps an FP32 state with a
                         compensated (Kahan) RK4 update; SAT weights and all
                         norms stay FP64 */
  long long nx, ny;   /* grid points per direction (ny ignored in 1D) */
  double xl[2], xr[2];/* domain [xl, xr]; h = (xr - xl)/(N - 1) as the demos */
  double a, b;        /* advection velocities (x, y) */
  const double* rho;  /* SBP_WAVE_VAR_2D: host array of nx*ny densities, (j,i) row-major */
  const double* K;    /* SBP_WAVE_VAR_2D: host array of nx*ny bulk moduli */
  void* stream;       /* cudaStream_t to run on, or NULL for a private stream */
  int device;         /* CUDA device ordinal */
  long long nz;       /* SBP_WAVE_3D: grid points in z (ignored otherwise) */
  double xl2, xr2;    /* SBP_WAVE_3D: z extent of the domain */
  /* Advection with a velocity at every point, the reference's velocity
   * callables a(i) (code/demo/advection/advection_rhs.h:12-51) and a(i,j),
   * b(i,j) (:155-393), whose inflow SAT takes tau from the velocity at the
   * boundary point (:94-119, :460-528): host arrays of nx (1D) or nx*ny (2D,
   * (j,i) row-major) velocities, copied at sbp_create. NULL: the constants a, b
   * (in 2D, a field given for one direction and not the other takes the
   * constant for the other everywhere). Single contexts only. */
  const double* a_field;
  const double* b_field;
} sbp_desc;

/* Creates a context: validates the description (N >= max(closure width,
 * 2*closure size) per direction), allocates the device state and scratch,
 * builds the TMA descriptors. Replaces the DMDA/AppCtx set-up of the demos'
 * main() (e.g. wave_eq_hom_sim.cpp:99-134). */
int sbp_create(const sbp_desc* desc, sbp_ctx** ctx);
int sbp_destroy(sbp_ctx* ctx);
const char* sbp_last_error(const sbp_ctx* ctx);
/* Scalars per grid point of the context's problem (4, 3, 2 or 1). */
int sbp_dofs(const sbp_ctx* ctx);
/* Doubles in one state in the AoS format: dofs * nx * ny (* nz). */
long long sbp_size(const sbp_ctx* ctx);

/* RHS callback body: dst = F(t, src) = matrix-free apply + boundary terms.
 * Replaces PetscErrorCode rhs_serial(TS, PetscReal t, Vec src, Vec dst, void*)
 * (code/demo/wave_hom/wave_eq_hom_sim.cpp:291-308; wave_eq_sim.cpp:291-308;
 * advection_1D_sim.cpp:212-228; advection_2D_sim.cpp:232-249;
 * reflection_sim.cpp:249-265). Synchronous. */
int sbp_rhs(sbp_ctx* ctx, double t, const double* src, double* dst, int where);

/* Matrix-free apply without boundary terms: wave_eq_hom_serial
 * (wave_eq_hom_rhs.h:365), wave_eq_serial (wave_eq_rhs.h:389),
 * advection_serial (advection_rhs.h:83,440), reflection_serial
 * (reflection_rhs.h:98). Synchronous. */
int sbp_apply(sbp_ctx* ctx, double t, const double* src, double* dst, int where);

/* Step count rule of the reference's RK4: round(t_end/dt) steps; dt is
 * replaced by t_end/steps when the two disagree by more than 1e-14
 * (code/include/time_stepping/time_stepping.h:104-109). */
long long sbp_rk4_nsteps(double t_end, double* dt);

/* Classical RK4 from t = 0 to t_end in place on v: the time-stepper entry
 * PetscErrorCode ts_rk4(DM, t_end, dt, Vec v, rhs, ctx)
 * (code/src/time_stepping/ts_rk.cpp:54-65), with the step rule above.
 * Copies v in, runs the CUDA-graph step loop, copies v out. Synchronous. */
int sbp_ts_rk4(sbp_ctx* ctx, double t_end, double dt, double* v, int where);

/* nsteps classical RK4 steps of size dt from t0, in place on v. Synchronous. */
int sbp_rk4(sbp_ctx* ctx, double t0, double dt, long long nsteps, double* v, int where);

/* Device-resident state: load / read back the context's state, and step it
 * without host transfers. sbp_rk4_resident only enqueues work on the
 * context's stream; sbp_synchronize waits and reports kernel errors. */
int sbp_set_state(sbp_ctx* ctx, const double* v, int where);
int sbp_get_state(sbp_ctx* ctx, double* v, int where);
int sbp_rk4_resident(sbp_ctx* ctx, double t0, double dt, long long nsteps);
int sbp_synchronize(sbp_ctx* ctx);

/* Norms of the resident state, reduced on the device in FP64.
 * error_l2 = sqrt(prod h) * ||state - exact||_2 and error_max = ||state - exact||_inf
 * over every component (error_l2 / error_max, code/include/util/vec_util.h:47-61);
 * exact is an AoS FP64 array (host or device). */
int sbp_error_norms(sbp_ctx* ctx, const double* exact, int where, double* error_l2, double* error_max);
/* Energy norm sqrt(sum_comp v^T H v) with the closure quadrature at both ends
 * of each direction (tensor product in 2D). The 1D form extends
 * H_central::get_norm_1D (code/include/sbpops/H_central.h:70-103), which on a
 * single rank applies the left closure weights only; the 2D form is
 * get_norm_2D, a TODO returning -1 in the reference (H_central.h:177-183). */
int sbp_hnorm(sbp_ctx* ctx, double* hnorm);

/* ---------------------------------------------------------------- adaptive RK45
 * Runge-Kutta-Fehlberg 4(5) with a basic step-size controller on the
 * context's device-resident state (FP64 contexts). Replaces ts_rk45
 * (code/include/time_stepping/ts_rk.h:15, code/src/time_stepping/ts_rk.cpp:41-52),
 * which runs PETSc's TSRK5F (Fehlberg's pair, advanced with the 5th-order
 * weights) under TSADAPTBASIC with TS_EXACTFINALTIME_MATCHSTEP and PETSc's
 * default options. The controller per attempted step h from time t:
 *   wlte = sqrt(mean over all scalars of ((u5 - u4) / (atol + rtol max(|u5|, |u4|)))^2),
 *   an entry with a zero tolerance contributing 0
 *   accept iff wlte <= 1; h' = h clip(safety' wlte^(-1/5), clip_lo, clip_hi)
 *   (safety' = safety, times reject_safety when this and the previous attempt
 *   failed), h' in [dt_min, dt_max]; with hmax = t_end - t: h' >= hmax -> hmax,
 *   otherwise 2 h' > hmax -> hmax/2 and 1.01 h' > hmax -> hmax.
 * The first attempt uses dt0 under the same landing rule. The run stops when
 * the attempt that lands on t_end is accepted (t = t_end exactly). */
typedef struct {
  double atol, rtol;            /* error tolerances (1e-4, 1e-4) */
  double safety, reject_safety; /* 0.9, 0.5 */
  double clip_lo, clip_hi;      /* bounds of the step change factor: 0.1, 10 */
  double dt_min, dt_max;        /* 1e-20, 1e50 */
  long long max_steps;          /* attempts (accepted + rejected) allowed: 1e7 */
  int max_reject;               /* rejections in a row allowed: 10 */
} sbp_rk45_opts;
typedef struct {
  long long accepted, rejected;
  double t;       /* time reached */
  double dt_next; /* step the controller proposes next */
  double wlte;    /* weighted error of the last attempt */
  int status;     /* 0 done; 1 step limit; 2 non-finite error; 3 rejections in a row */
} sbp_rk45_stats;
void sbp_rk45_default_opts(sbp_rk45_opts* opts);
/* From t0 to t_end on the resident state; opts NULL = defaults, stats may be
 * NULL. Synchronous. SBP_ERR_DIVERGED when the controller stopped early (the
 * state then holds the last accepted step). */
int sbp_rk45_resident(sbp_ctx* ctx, double t0, double t_end, double dt0, const sbp_rk45_opts* opts,
                      sbp_rk45_stats* stats);
/* ts_rk45(da, t_end, dt, v, rhs, ctx): from t = 0, default options, in place on v. */
int sbp_ts_rk45(sbp_ctx* ctx, double t_end, double dt, double* v, int where);

/* The context's CUDA stream (cudaStream_t) and the number of kernels the
 * context has launched so far (graph replays count each kernel node). */
int sbp_get_stream(const sbp_ctx* ctx, void** stream);
long long sbp_launch_count(const sbp_ctx* ctx);

/* Failure detection (no counterpart in the reference, whose MPI ranks have
 * no device waits). Every mbarrier wait in the 2D wave stage kernels is
 * bounded by %globaltimer; a wait that runs out sets the context's error word,
 * the kernel lets its copies in flight land and returns, and the next
 * sbp_synchronize (or the synchronous entry point that launched it) returns
 * SBP_ERR_DEVICE and clears the word: the context stays usable.
 * sbp_set_wait_limit: the limit in ns (default 200 ms; 0 restores it); drops
 *   the context's captured step graphs, which carry the old limit.
 * sbp_test_drop_tile: test aid for that path. The next sbp_rhs / sbp_apply of
 *   a 2D wave context issues no load for tile `tile` (row-major index of the
 *   stage kernel's tiles), so the wait for it runs out and the call returns
 *   SBP_ERR_DEVICE. Nothing faults or hangs; never applies to RK4 steps. */
int sbp_set_wait_limit(sbp_ctx* ctx, long long ns);
int sbp_test_drop_tile(sbp_ctx* ctx, long long tile);

/* Measured FP64 FMA throughput of the current device in DFMA/s (a
 * 1-second-scale probe). No counterpart in the reference; used to state the
 * FP64 ALU roof beside the HBM roof. */
int sbp_probe_dfma_rate(int device, double* dfma_per_s);

/* ---------------------------------------------------------------- batches
 * Many independent instances of uneven size, order and coefficients
 * advanced together: 2D waves (rho = 1, K = c^2) and 2D advection. No
 * counterpart in the reference, which runs one grid per process; each
 * instance computes what a single-instance context of the same problem
 * computes (the same per-point arithmetic). Per order, one persistent stage
 * kernel walks a tile list over all wave instances; the step loop runs in
 * CUDA graphs of 100 steps; each instance has its own time step. */
typedef struct sbp_batch sbp_batch;
typedef struct {
  int problem;        /* SBP_WAVE_HOM_2D (wave speed c) or SBP_ADVECTION_2D (velocity a, b) */
  int order;          /* 2, 4 or 6 */
  int bc;             /* wave: SBP_BC_REFERENCE (free surface) or SBP_BC_CHARACTERISTIC */
  long long nx, ny;
  double xl[2], xr[2];
  double c;           /* wave speed (rho = 1, K = c^2) */
  double a, b;        /* advection velocity */
  double dt;          /* this instance's time step */
} sbp_instance;

int sbp_batch_create(const sbp_instance* list, int count, int precision, int device, void* stream,
                     sbp_batch** batch);
int sbp_batch_destroy(sbp_batch* batch);
const char* sbp_batch_last_error(const sbp_batch* batch); /* NULL: last failed sbp_batch_create */
/* State of instance `index` in the reference's AoS layout (host or device). */
int sbp_batch_set_state(sbp_batch* batch, int index, const double* v, int where);
int sbp_batch_get_state(sbp_batch* batch, int index, double* v, int where);
/* nsteps RK4 steps of every instance (each with its own dt); enqueues only. */
int sbp_batch_rk4_resident(sbp_batch* batch, long long nsteps);
int sbp_batch_synchronize(sbp_batch* batch);
/* Picks the kernel configuration of each (order, problem) group -- tile rows,
 * compute warps, ring depth, CTAs per SM (and, for FP64 waves, the fixed-point
 * stencil kernel or FP64 taps), from a table of four per kind and
 * precision -- by timing each group's middle stage on this batch, then a few
 * whole steps with those choices and with every group on each table entry,
 * keeping the fastest; results are cached in the flat JSON file cache_path
 * (NULL: no cache). Call between steps: the states are saved before the trial
 * steps and restored after them (one extra state buffer, freed on return). */
int sbp_batch_autotune(sbp_batch* batch, const char* cache_path);
/* Tile rows of the order's wave group (0: no wave instance of that order). */
int sbp_batch_tile_height(const sbp_batch* batch, int order);
/* cfg[0..4] = tile rows, compute warps, ring depth, CTAs per SM and converter
 * warps (FP64 waves: the fixed-point stencil kernel; 0: FP64 taps) of the group
 * of `order` and `problem` (SBP_WAVE_HOM_2D or SBP_ADVECTION_2D); zeros for an
 * empty group. */
int sbp_batch_kernel_config(const sbp_batch* batch, int order, int problem, int* cfg);
/* Makes entry `index` (0..3) of the group's configuration table the one it runs
 * (what sbp_batch_autotune does with the fastest). Call between steps. */
int sbp_batch_select_config(sbp_batch* batch, int order, int problem, int index);
int sbp_batch_get_stream(const sbp_batch* batch, void** stream);
long long sbp_batch_points(const sbp_batch* batch);       /* grid points over all instances */
long long sbp_batch_launch_count(const sbp_batch* batch); /* kernels launched so far */

/* ---------------------------------------------------------------- decomposed grid
 * One SBP_WAVE_HOM_2D grid (FP64) split into px x py subdomains, each with its
 * own state and R ghost lines per side, on one device. Replaces the reference's
 * decomposed path: rhs_local / rhs_all per DMDA block
 * (code/include/partitioned_rhs/rhs.h:97-181, 183-360) with the VecScatter ghost
 * update before each RHS (code/src/scatter/scatter_ctx.cpp:149-211), here fused
 * into the RK4 stage kernels: each stage writes its edge values into the
 * neighbours' ghost lines as well (a halo kernel runs once per call, for the
 * state it starts from). Subdomain widths are
 * floor(N*(b+1)/p) - floor(N*b/p) >= the closure width (2 / 6 / 9 points for
 * orders 2 / 4 / 6) and the whole grid at least sbp_create's minimum size,
 * else SBP_ERR_INVALID; other problems or FP32:
 * SBP_ERR_UNSUPPORTED. Results equal sbp_create's single grid to rounding.
 * States are the full grid's AoS arrays (as sbp_set_state). Synchronous. */
typedef struct sbp_decomp sbp_decomp;
int sbp_decomp_create(const sbp_desc* desc, int px, int py, sbp_decomp** dec);
int sbp_decomp_destroy(sbp_decomp* dec);
const char* sbp_decomp_last_error(const sbp_decomp* dec); /* NULL: the last failed sbp_decomp_create */
int sbp_decomp_set_state(sbp_decomp* dec, const double* state, int where);
int sbp_decomp_get_state(sbp_decomp* dec, double* state, int where);
/* dst = F(src) (the system is autonomous): halo exchange, then the RHS of every subdomain. */
int sbp_decomp_rhs(sbp_decomp* dec, const double* src, double* dst, int where);
/* nsteps classical RK4 steps of the resident state; every stage also fills the ghost lines its
 * successor reads. The steps run as CUDA graphs of up to 50 steps, one per chunk length,
 * kept across calls until dt changes. */
int sbp_decomp_rk4_resident(sbp_decomp* dec, double dt, long long nsteps);

/* ---------------------------------------------------------------- learned correction
 * A 4-layer 3x3 convolutional network (24 -> 32 -> 32 -> 32 -> 3 channels,
 * ReLU) that corrects a coarse solve; no counterpart in the reference.
 * Inputs and outputs are device arrays, NHWC FP32 (features: sbp_cnn_features;
 * outputs: corrections of Z u, Z v, p in units of a scale, sbp_cnn_correct).
 * Inside: BF16 activations and weights, FP32 accumulation in tensor memory
 * (tcgen05 convolutions), FP32 master weights, Adam. Parameters as one FP32
 * vector: per layer the weights [cout][9][cin] (channels padded: layer 1 cin 32
 * of which 24 real, layer 4 cout 16 of which 3 real) then the bias [cout].
 * forward / gradients / train_step are synchronous; a convolution whose bounded
 * wait for its tiles ran out makes them return SBP_ERR_DEVICE (the word is
 * cleared: the network stays usable). */
typedef struct sbp_cnn sbp_cnn;
int sbp_cnn_create(int height, int width, int max_batch, int device, void* stream, sbp_cnn** cnn);
int sbp_cnn_destroy(sbp_cnn* cnn);
const char* sbp_cnn_last_error(const sbp_cnn* cnn); /* NULL: last failed sbp_cnn_create */
long long sbp_cnn_param_count(void);
/* He-normal weights for layers 1-3 from `seed`, zero output layer, zero biases, Adam reset. */
int sbp_cnn_init(sbp_cnn* cnn, unsigned long long seed);
int sbp_cnn_get_params(sbp_cnn* cnn, float* host, long long n);
int sbp_cnn_set_params(sbp_cnn* cnn, const float* host, long long n);
int sbp_cnn_forward(sbp_cnn* cnn, const float* x, int batch, float* out);
/* Gradients of the mean squared error (host vector in the parameter layout, may be NULL). */
int sbp_cnn_gradients(sbp_cnn* cnn, const float* x, const float* target, int batch, float* grad, long long n,
                      float* loss);
/* One Adam step (beta 0.9 / 0.999) on the mean squared error of a batch;
 * weights are trained, biases keep their values (zero after sbp_cnn_init). */
int sbp_cnn_train_step(sbp_cnn* cnn, const float* x, const float* target, int batch, float lr, float* loss);
/* Device helpers of the corrected solve on a layered grid (ny = blocks x
 * block_rows rows of nx points, nx and block_rows >= 5, AoS FP64 u, v, p;
 * rho, K per point). Features (24 per point, inv_scale = 1/s), with
 * q = (Z u, Z v, p), Z = sqrt(rho K), computed in FP64 and divided by s:
 * undivided second differences of q along x (3) and along y within the
 * point's block (3), fourth differences along x (3) and y (3), then the same
 * twelve times +1 in block 0 and -1 above. Centres are clamped one (second
 * differences) or two (fourth) points in from an edge.
 * sbp_cnn_correct: state += scale * (delta_0 / Z, delta_1 / Z, delta_2). */
int sbp_cnn_features(const double* state, const double* rho, const double* K, int nx, int ny, int block_rows,
                     double inv_scale, float* x, void* stream);
int sbp_cnn_correct(double* state, const float* delta, const double* rho, const double* K, long long npts,
                    double scale, void* stream);
long long sbp_cnn_launch_count(const sbp_cnn* cnn);

/* PETSc binary Vec files (host-side I/O): the format VecView writes on a
 * binary viewer, as the reference's write_vector_to_binary does
 * (code/src/util/io_util.cpp:4-14): big-endian int32 classid 1211214,
 * big-endian int32 length, big-endian doubles. A single-rank DMDA vector is
 * written in the AoS order of this library's boundary arrays.
 * sbp_read_petsc_vec: with v == NULL only *n is set; fails if *n > capacity. */
int sbp_write_petsc_vec(const char* path, const double* v, long long n);
int sbp_read_petsc_vec(const char* path, double* v, long long capacity, long long* n);

/* RHS of the 2D acoustic wave system (rho = K = 1, FP64) that allocates no
 * device memory. It has no counterpart in the reference.
 *
 * sbp_rhs needs a context, and a context's staging buffers come from
 * cudaMalloc. Some callers cannot allocate: a host framework that owns all
 * device memory through its own pool and forbids plugins to call cudaMalloc,
 * or a caller in a latency-bound loop that cannot take cudaMalloc's implicit
 * device synchronisation. This entry point computes what sbp_rhs computes for
 * that problem (free-surface or characteristic SAT, orders 2/4/6) with its
 * scratch in one fixed-size static device array that every GPU loading the
 * library holds until exit: 6 * SBP_NOALLOC_MAX_PLANE doubles (3 MiB) plus an
 * error word.
 *
 * desc: problem SBP_WAVE_HOM_2D, precision SBP_FP64, order, bc, nx, ny, xl, xr,
 *       device, stream (NULL = the legacy default stream); rho, K, a, b unused.
 * src, dst: caller-owned DEVICE arrays of nx*ny*3 doubles in the reference's
 *       AoS layout. Synchronous on desc->stream.
 * Limit: roundup(nx, 64) * ny <= SBP_NOALLOC_MAX_PLANE (e.g. 256 x 256);
 *       larger grids return SBP_ERR_TOO_LARGE before any GPU work.
 * Sharing: all calls on a device use the same array; the error word is
 *       cleared by each call, the rest is overwritten. Calls whose GPU work
 *       overlaps (other streams or threads) race on the array: serialise them.
 * First call on a device: does a one-time set-up on that device (the array's
 *       device address, the kernels' shared-memory opt-in); make it before
 *       any stream capture. Later calls look the address up again and redo
 *       the set-up if it moved (after cudaDeviceReset).
 * Every call is synchronous: it waits on desc->stream for its own work and
 *       reads the kernel's error word back to the host before returning.
 *       The calling thread's current device is restored on return. */
#define SBP_NOALLOC_MAX_PLANE 65536
int sbp_wave_rhs_noalloc(const sbp_desc* desc, double t, const double* src, double* dst);

#ifdef __cplusplus
}
#endif
#endif /* SBPGPU_H */
