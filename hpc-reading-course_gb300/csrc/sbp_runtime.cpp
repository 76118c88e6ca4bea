// sbp_runtime.cpp -- host runtime behind the C ABI (include/sbpgpu.h):
// device-resident SoA state, TMA descriptors, the RK4 stage sequence and its
// CUDA-graph step loop, the layout conversion at the reference boundary, and
// the FP64 norms.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <string>

#include "../../include/sbpgpu.h"
#include "launch.h"
#include "sbp_ops.h"

using namespace sbp;

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

bool is_wave(int problem) {
  return problem == SBP_WAVE_HOM_2D || problem == SBP_WAVE_MMS_2D || problem == SBP_WAVE_VAR_2D ||
         problem == SBP_WAVE_2BLOCK_2D;
}
bool has_fields(int problem) { return problem == SBP_WAVE_VAR_2D || problem == SBP_WAVE_2BLOCK_2D; }
bool is_2d(int problem) { return is_wave(problem) || problem == SBP_ADVECTION_2D; }
int dofs_of(int problem) {
  if (problem == SBP_WAVE_3D) return 4;
  if (is_wave(problem)) return 3;
  return problem == SBP_REFLECTION_1D ? 2 : 1;
}

}  // namespace

struct sbp_ctx {
  sbp_desc d{};
  int dofs = 0;
  bool fp32 = false, two_d = false, wave = false, time_dependent = false;
  bool three_d = false;  // SBP_WAVE_3D: nz slabs of ny rows; row-generic kernels see ny * nz rows
  long long nx = 0, ny = 1, nz = 1, pitch = 0, plane = 0, npts = 0, nscalar = 0;
  int ysplit = 0;  // two-block problems: first row of the upper block
  size_t es = 8;
  double hix = 1, hiy = 1, hx = 1, hy = 1, hiz = 1, hz = 1;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // device buffers: SoA planes (dofs * plane elements of T each)
  void *un = nullptr, *acc = nullptr, *wa = nullptr, *wb = nullptr, *comp = nullptr;
  double* io = nullptr;       // AoS FP64 staging, nscalar
  double* partial = nullptr;  // reduction scratch, 2 * kReduceBlocks
  double* red = nullptr;      // reduction result, 4
  void *rinv = nullptr, *kmod = nullptr;     // WAVE_VAR: T planes
  void *va = nullptr, *vb = nullptr;         // advection with velocity fields: T planes (pitched)
  double *va64 = nullptr, *vb64 = nullptr;   // the same in FP64, nx*ny row-major (SAT)
  double *rho64 = nullptr, *k64 = nullptr;   // WAVE_VAR: nx*ny FP64
  int* err = nullptr;
  int* sched = nullptr;  // the wave stage kernels' dynamic tile queue (2 ints, zero between launches)
  WaveMaps maps_un{}, maps_wa{}, maps_wb{};
  // adaptive RK45 (FP64; allocated on first use)
  double* rk_k[6] = {};
  double* rk_unew = nullptr;
  Rk45Ctrl* rk_ctrl = nullptr;
  double rk_atol = 0, rk_rtol = 0;  // tolerances baked into the fused wave stages
  cudaGraphExec_t rk_graph = nullptr;
  std::map<long long, cudaGraphExec_t> graphs;
  double graph_dt = 0.0;
  long long launches = 0;
  unsigned long long wait_ns = 0;  // limit of the wave stage kernels' bounded waits (0: the kernel default)
  int drop_tile = 0;               // test aid: tile + 1 whose load the next RHS evaluation skips
  std::string msg;
};

namespace {

// Message of the last sbp_create failure on this thread (no context exists then).
thread_local std::string g_create_error;

int fail(sbp_ctx* c, int code, const std::string& m) {
  if (c) c->msg = m;
  return code;
}

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(ctx, SBP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
void fill_taps(DirTaps<T>& t, int order, double scale) {
  const ops::Operator& op = ops::get(order);
  std::memset(&t, 0, sizeof(t));
  for (int s = 0; s < op.width; s++) t.taps[s] = (T)(scale * op.interior[s]);
  for (int r = 0; r < op.cls_sz; r++)
    for (int s = 0; s < op.cls_width; s++) t.cls[r][s] = (T)(scale * op.closure[r][s]);
}

int wave_kind(const sbp_ctx* ctx) {
  if (ctx->d.problem == SBP_WAVE_HOM_2D) return WK_HOM;
  return has_fields(ctx->d.problem) ? WK_VAR : WK_MMS;
}

// Encodes one 3D tensor map (x, y, component) over a state buffer of the context.
int encode_map(sbp_ctx* ctx, void* base, const cuuint32_t box[3], CUtensorMap* out) {
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return fail(ctx, SBP_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const cuuint64_t dims[3] = {(cuuint64_t)ctx->nx, (cuuint64_t)ctx->ny, 3};
  const cuuint64_t strides[2] = {(cuuint64_t)(ctx->pitch * ctx->es), (cuuint64_t)(ctx->plane * ctx->es)};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUtensorMapDataType dt = ctx->fp32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  CUresult r = enc(out, dt, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(ctx, SBP_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string(r));
  return SBP_OK;
}

// Stencil-tile maps of a stage-input buffer plus the point maps of u^n, acc
// and the Kahan term (the same for every input buffer).
int make_maps(sbp_ctx* ctx, void* base, WaveMaps& m) {
  const int R = ctx->d.order / 2;
  const int hxa = 16 / (int)ctx->es;
  const int HX = (R + hxa - 1) / hxa * hxa, HY = R;
  const int TY = wave_tile_height((int)ctx->es, wave_kind(ctx));
  const cuuint32_t boxP[3] = {(cuuint32_t)(kWaveTX + 2 * HX), (cuuint32_t)(TY + 2 * HY), 1};
  const cuuint32_t boxU[3] = {(cuuint32_t)(kWaveTX + 2 * HX), (cuuint32_t)TY, 1};
  const cuuint32_t boxV[3] = {(cuuint32_t)kWaveTX, (cuuint32_t)(TY + 2 * HY), 1};
  const cuuint32_t boxPt[3] = {(cuuint32_t)kWaveTX, (cuuint32_t)TY, 3};
  int rc;
  if ((rc = encode_map(ctx, base, boxP, &m.p)) || (rc = encode_map(ctx, base, boxU, &m.u)) ||
      (rc = encode_map(ctx, base, boxV, &m.v)) || (rc = encode_map(ctx, ctx->un, boxPt, &m.n)) ||
      (rc = encode_map(ctx, ctx->acc, boxPt, &m.a)) ||
      (rc = encode_map(ctx, ctx->comp ? ctx->comp : ctx->acc, boxPt, &m.c)))
    return rc;
  if (!ctx->rinv) {
    m.k = m.p;  // no coefficient fields: the map is never used
    return SBP_OK;
  }
  // [1/rho | K]: two planes at rinv (kmod follows it), as a 2-component point box
  EncodeTiledFn enc = encode_tiled();
  const cuuint64_t dims[3] = {(cuuint64_t)ctx->nx, (cuuint64_t)ctx->ny, 2};
  const cuuint64_t strides[2] = {(cuuint64_t)(ctx->pitch * ctx->es), (cuuint64_t)(ctx->plane * ctx->es)};
  const cuuint32_t estr[3] = {1, 1, 1};
  const cuuint32_t boxK[3] = {(cuuint32_t)kWaveTX, (cuuint32_t)TY, 2};
  const CUtensorMapDataType dt = ctx->fp32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  if (enc(&m.k, dt, 3, ctx->rinv, dims, strides, boxK, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return fail(ctx, SBP_ERR_CUDA, "cuTensorMapEncodeTiled failed for the coefficient planes");
  return SBP_OK;
}

// Stage-independent kernel parameters.
template <typename T>
WaveParams<T> wave_params(sbp_ctx* ctx) {
  WaveParams<T> p;
  std::memset(&p, 0, sizeof(p));
  p.nx = (int)ctx->nx;
  p.ny = (int)ctx->ny;
  p.pitch = ctx->pitch;
  p.plane = ctx->plane;
  p.rinv = (const T*)ctx->rinv;
  p.kmod = (const T*)ctx->kmod;
  p.rho64 = ctx->rho64;
  p.k64 = ctx->k64;
  fill_taps<T>(p.dx, ctx->d.order, -ctx->hix);
  fill_taps<T>(p.dy, ctx->d.order, -ctx->hiy);
  const double hi0 = ops::get(ctx->d.order).hinv0;
  p.bwx = ctx->hix * hi0;
  p.bwy = ctx->hiy * hi0;
  p.bc = ctx->d.bc == SBP_BC_CHARACTERISTIC ? BC_CHARACTERISTIC : BC_FREE_SURFACE;
  p.ysplit = ctx->ysplit;
  p.xl0 = ctx->d.xl[0];
  p.xl1 = ctx->d.xl[1];
  p.hix = ctx->hix;
  p.hiy = ctx->hiy;
  p.err = ctx->err;
  return p;
}

template <typename T>
LineParams<T> line_params(sbp_ctx* ctx) {
  LineParams<T> p;
  std::memset(&p, 0, sizeof(p));
  p.nx = (int)ctx->nx;
  p.ny = (int)ctx->ny;
  p.pitch = ctx->pitch;
  p.plane = ctx->plane;
  const double hi0 = ops::get(ctx->d.order).hinv0;
  const double a = ctx->d.a, b = ctx->d.b;
  if (ctx->d.problem == SBP_REFLECTION_1D) {
    fill_taps<T>(p.dx, ctx->d.order, ctx->hix);
  } else if (ctx->va) {  // velocity fields: the kernel forms -(a(x) D1x + b(x) D1y)
    fill_taps<T>(p.dx, ctx->d.order, ctx->hix);
    fill_taps<T>(p.dy, ctx->d.order, ctx->hiy);
    p.va = (const T*)ctx->va;
    p.vb = (const T*)ctx->vb;
    p.va64 = ctx->va64;
    p.vb64 = ctx->vb64;
    p.bw[0] = ctx->hix * hi0;
    p.bw[1] = ctx->hiy * hi0;
  } else {
    fill_taps<T>(p.dx, ctx->d.order, -a * ctx->hix);
    fill_taps<T>(p.dy, ctx->d.order, -b * ctx->hiy);
    // SAT_bc_* (advection_rhs.h:94-119, 460-528): 0.5 * tau * hi * HI[0]
    p.sat[0] = 0.5 * (-0.5 * (a + std::fabs(a))) * (ctx->hix * hi0);
    p.sat[1] = 0.5 * (-0.5 * (b + std::fabs(b))) * (ctx->hiy * hi0);
    p.sat[2] = 0.5 * (0.5 * (a - std::fabs(a))) * (ctx->hix * hi0);
    p.sat[3] = 0.5 * (0.5 * (b - std::fabs(b))) * (ctx->hiy * hi0);
  }
  p.bc = 1;
  p.compensated = ctx->fp32 ? 1 : 0;
  p.err = ctx->err;
  return p;
}

int line_kind(const sbp_ctx* ctx) {
  return ctx->d.problem == SBP_ADVECTION_1D ? LK_ADV1D : (ctx->d.problem == SBP_REFLECTION_1D ? LK_REFL1D : LK_ADV2D);
}

// Launches one kernel of the stage sequence. `in` is the state the RHS is
// evaluated on; `in_maps` its TMA descriptors (2D wave only).
template <typename T>
int launch_stage(sbp_ctx* ctx, int stage, int rk, double t, double dt, void* in, const WaveMaps* in_maps,
                 void* kout, int bc_on, const Rk45Ctrl* ctl = nullptr, double tc = 0.0) {
  T c_acc = 0, c_w = 0;
  if (stage == ST_FIRST) {
    c_acc = (T)(dt / 6);
    c_w = (T)(0.5 * dt);
  } else if (stage == ST_MID) {
    c_acc = (T)(dt / 3);
    c_w = (T)(rk == 2 ? 0.5 * dt : dt);
  } else if (stage == ST_LAST) {
    c_acc = (T)(dt / 6);
  }
  void* wout = (rk == 1 || rk == 3) ? ctx->wa : ctx->wb;
  if (ctx->wave) {
    WaveParams<T> p = wave_params<T>(ctx);
    p.in = (const T*)in;
    p.un = (T*)ctx->un;
    p.acc = (T*)ctx->acc;
    p.wout = (T*)wout;
    p.kout = (T*)kout;
    p.comp = (T*)ctx->comp;
    p.c_acc = c_acc;
    p.c_w = c_w;
    p.t = t;
    p.wait_ns = ctx->wait_ns;
    p.sched = ctx->sched;
    if constexpr (sizeof(T) == 8) set_fixed_scales(p, ctx->d.order, ctx->hix, ctx->hiy);
    if (stage == ST_RHS) {  // a direct launch (RHS evaluation), never a captured one
      p.test_drop_tile = ctx->drop_tile;
      ctx->drop_tile = 0;
    }
    if (ctl) {  // adaptive integrator: stage time and stop flag from device memory
      p.tctl = &ctl->t;
      p.tc = tc;
      p.skip = &ctl->done;
    }
    if (!bc_on) p.bc = BC_NONE;
    CK(launch_wave<T>(ctx->d.order, wave_kind(ctx), stage, *in_maps, p, ctx->stream));
  } else if (ctx->three_d) {
    Wave3Params<T> p;
    std::memset(&p, 0, sizeof(p));
    p.nx = (int)ctx->nx;
    p.ny = (int)ctx->ny;
    p.nz = (int)ctx->nz;
    p.pitch = ctx->pitch;
    p.slab = ctx->pitch * ctx->ny;
    p.plane = ctx->plane;
    p.in = (const T*)in;
    p.un = (T*)ctx->un;
    p.acc = (T*)ctx->acc;
    p.wout = (T*)wout;
    p.kout = (T*)kout;
    p.comp = (T*)ctx->comp;
    fill_taps<T>(p.dx, ctx->d.order, -ctx->hix);
    fill_taps<T>(p.dy, ctx->d.order, -ctx->hiy);
    fill_taps<T>(p.dz, ctx->d.order, -ctx->hiz);
    const double hi0 = ops::get(ctx->d.order).hinv0;
    p.bw[0] = ctx->hix * hi0;
    p.bw[1] = ctx->hiy * hi0;
    p.bw[2] = ctx->hiz * hi0;
    p.bc = !bc_on ? BC_NONE : (ctx->d.bc == SBP_BC_CHARACTERISTIC ? BC_CHARACTERISTIC : BC_FREE_SURFACE);
    p.compensated = ctx->fp32 ? 1 : 0;
    p.c_acc = c_acc;
    p.c_w = c_w;
    if (ctl) p.skip = &ctl->done;
    CK(launch_wave3d<T>(ctx->d.order, stage, p, ctx->stream));
  } else {
    LineParams<T> p = line_params<T>(ctx);
    p.in = (const T*)in;
    p.un = (T*)ctx->un;
    p.acc = (T*)ctx->acc;
    p.wout = (T*)wout;
    p.kout = (T*)kout;
    p.comp = (T*)ctx->comp;
    p.c_acc = c_acc;
    p.c_w = c_w;
    p.bc = bc_on;
    if (ctl) p.skip = &ctl->done;
    CK(launch_line<T>(ctx->d.order, line_kind(ctx), stage, p, ctx->stream));
  }
  ctx->launches++;
  return SBP_OK;
}

// One classical RK4 step on the resident state (time_stepping.h:127-142):
// stage 1 reads u^n and writes acc, wa; stage 2 reads wa, writes acc, wb;
// stage 3 reads wb, writes acc, wa; stage 4 reads wa, acc and writes u^{n+1}.
template <typename T>
int enqueue_step(sbp_ctx* ctx, double t, double dt) {
  int rc;
  if ((rc = launch_stage<T>(ctx, ST_FIRST, 1, t, dt, ctx->un, &ctx->maps_un, nullptr, 1))) return rc;
  if ((rc = launch_stage<T>(ctx, ST_MID, 2, t + 0.5 * dt, dt, ctx->wa, &ctx->maps_wa, nullptr, 1))) return rc;
  if ((rc = launch_stage<T>(ctx, ST_MID, 3, t + 0.5 * dt, dt, ctx->wb, &ctx->maps_wb, nullptr, 1))) return rc;
  return launch_stage<T>(ctx, ST_LAST, 4, t + dt, dt, ctx->wa, &ctx->maps_wa, nullptr, 1);
}

void drop_graphs(sbp_ctx* ctx) {
  for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
  ctx->graphs.clear();
}

template <typename T>
int run_chunk_graph(sbp_ctx* ctx, long long steps, double dt) {
  if (ctx->graph_dt != dt) {
    drop_graphs(ctx);
    ctx->graph_dt = dt;
  }
  auto it = ctx->graphs.find(steps);
  if (it == ctx->graphs.end()) {
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = ctx->launches;
    int rc = SBP_OK;
    for (long long s = 0; s < steps && rc == SBP_OK; s++) rc = enqueue_step<T>(ctx, 0.0, dt);
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
    ctx->launches = before;  // captured, not yet run
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    CK(ce);
    cudaGraphExec_t ex = nullptr;
    cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    CK(ie);
    it = ctx->graphs.emplace(steps, ex).first;
  }
  CK(cudaGraphLaunch(it->second, ctx->stream));
  ctx->launches += 4 * steps;
  return SBP_OK;
}

template <typename T>
int rk4_resident_t(sbp_ctx* ctx, double t0, double dt, long long nsteps) {
  if (ctx->time_dependent) {  // stage times change every step: direct launches
    double t = t0;
    for (long long s = 0; s < nsteps; s++) {
      int rc = enqueue_step<T>(ctx, t, dt);
      if (rc) return rc;
      t = t + dt;
    }
    return SBP_OK;
  }
  const long long chunk = 50;
  long long left = nsteps;
  while (left >= chunk) {
    int rc = run_chunk_graph<T>(ctx, chunk, dt);
    if (rc) return rc;
    left -= chunk;
  }
  if (left > 0) return run_chunk_graph<T>(ctx, left, dt);
  return SBP_OK;
}

int check_device_errors(sbp_ctx* ctx) {
  int h = 0;
  CK(cudaMemcpyAsync(&h, ctx->err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (h) {
    cudaMemsetAsync(ctx->err, 0, sizeof(int), ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    return fail(ctx, SBP_ERR_DEVICE, (h & ERR_TMA_TIMEOUT) ? "a TMA tile wait timed out in a stage kernel"
                                                           : "a kernel reported an error");
  }
  return SBP_OK;
}

// AoS FP64 input (host or device) -> a device AoS pointer.
int stage_in(sbp_ctx* ctx, const double* src, int where, const double** dev) {
  if (!src) return fail(ctx, SBP_ERR_INVALID, "null array");
  if (where == SBP_DEVICE) {
    *dev = src;
    return SBP_OK;
  }
  if (where != SBP_HOST) return fail(ctx, SBP_ERR_INVALID, "where must be SBP_HOST or SBP_DEVICE");
  CK(cudaMemcpyAsync(ctx->io, src, ctx->nscalar * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  *dev = ctx->io;
  return SBP_OK;
}

int pack_into(sbp_ctx* ctx, const double* aos, void* soa) {
  if (ctx->fp32)
    CK(launch_pack<float>(aos, (float*)soa, (int)ctx->nx, (int)(ctx->ny * ctx->nz), ctx->dofs, ctx->pitch, ctx->plane,
                          ctx->stream));
  else
    CK(launch_pack<double>(aos, (double*)soa, (int)ctx->nx, (int)(ctx->ny * ctx->nz), ctx->dofs, ctx->pitch, ctx->plane,
                           ctx->stream));
  ctx->launches++;
  return SBP_OK;
}

int unpack_to(sbp_ctx* ctx, const void* soa, double* dst, int where) {
  if (!dst) return fail(ctx, SBP_ERR_INVALID, "null array");
  double* out = (where == SBP_DEVICE) ? dst : ctx->io;
  if (ctx->fp32)
    CK(launch_unpack<float>((const float*)soa, out, (int)ctx->nx, (int)(ctx->ny * ctx->nz), ctx->dofs, ctx->pitch,
                            ctx->plane,
                            ctx->stream));
  else
    CK(launch_unpack<double>((const double*)soa, out, (int)ctx->nx, (int)(ctx->ny * ctx->nz), ctx->dofs, ctx->pitch,
                             ctx->plane,
                             ctx->stream));
  ctx->launches++;
  if (where != SBP_DEVICE)
    CK(cudaMemcpyAsync(dst, ctx->io, ctx->nscalar * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  return SBP_OK;
}

int rhs_impl(sbp_ctx* ctx, double t, const double* src, double* dst, int where, int bc_on) {
  if (!ctx) return SBP_ERR_INVALID;
  CK(cudaSetDevice(ctx->d.device));
  const double* dev = nullptr;
  int rc;
  if ((rc = stage_in(ctx, src, where, &dev))) return rc;
  if ((rc = pack_into(ctx, dev, ctx->wa))) return rc;
  if (ctx->fp32)
    rc = launch_stage<float>(ctx, ST_RHS, 0, t, 0.0, ctx->wa, &ctx->maps_wa, ctx->wb, bc_on);
  else
    rc = launch_stage<double>(ctx, ST_RHS, 0, t, 0.0, ctx->wa, &ctx->maps_wa, ctx->wb, bc_on);
  if (rc) return rc;
  if ((rc = unpack_to(ctx, ctx->wb, dst, where))) return rc;
  return check_device_errors(ctx);
}

// ---------------------------------------------------------------- adaptive RK45
Rk45Buffers rk45_buffers(sbp_ctx* ctx) {
  Rk45Buffers b;
  std::memset(&b, 0, sizeof(b));
  b.nx = (int)ctx->nx;
  b.ny = (int)(ctx->ny * ctx->nz);  // rows per component plane
  b.dofs = ctx->dofs;
  b.pitch = ctx->pitch;
  b.plane = ctx->plane;
  b.u = (double*)ctx->un;
  b.w = (double*)ctx->wa;
  for (int s = 0; s < 6; s++) b.k[s] = ctx->rk_k[s];
  b.unew = ctx->rk_unew;
  b.partial = ctx->partial;
  return b;
}

int rk45_prepare(sbp_ctx* ctx) {
  if (ctx->rk_ctrl) return SBP_OK;
  const size_t bytes = (size_t)ctx->dofs * ctx->plane * sizeof(double);
  for (int s = 0; s < 6; s++) CK(cudaMalloc((void**)&ctx->rk_k[s], bytes));
  CK(cudaMalloc((void**)&ctx->rk_unew, bytes));
  CK(cudaMemsetAsync(ctx->rk_unew, 0, bytes, ctx->stream));  // row padding stays zero
  CK(cudaMalloc((void**)&ctx->rk_ctrl, sizeof(Rk45Ctrl)));
  return SBP_OK;
}

// Fehlberg stage times c_s (the abscissae of the tableau in rk45.cu).
constexpr double kRkfC[6] = {0.0, 1.0 / 4, 3.0 / 8, 12.0 / 13, 1.0, 1.0 / 2};

// Fused Fehlberg stage s (1..6) of the 2D wave kernel: k_s from the stage input
// `in`, then the next stage input into `wout` (s < 6) or the candidate solution
// and one error partial per CTA (s = 6). Inputs alternate un -> wa -> wb -> wa ...
// so that no CTA overwrites halo rows another CTA is still reading.
int launch_rkf_wave_stage(sbp_ctx* ctx, int s, void* in, const WaveMaps* in_maps, void* wout) {
  WaveParams<double> p = wave_params<double>(ctx);
  const Rk45Ctrl* ctl = ctx->rk_ctrl;
  p.in = (const double*)in;
  p.wout = (double*)wout;
  p.tctl = &ctl->t;
  p.tc = kRkfC[s - 1];
  p.skip = &ctl->done;
  for (int j = 0; j < 6; j++) p.rkk[j] = ctx->rk_k[j];
  p.rku = (const double*)ctx->un;
  p.rkunew = ctx->rk_unew;
  p.rkpart = ctx->partial;
  p.rkatol = ctx->rk_atol;
  p.rkrtol = ctx->rk_rtol;
  p.wait_ns = ctx->wait_ns;
  CK(launch_wave<double>(ctx->d.order, wave_kind(ctx), ST_RKF1 + s - 1, *in_maps, p, ctx->stream));
  ctx->launches++;
  return SBP_OK;
}

// CTAs of the persistent wave kernel (as launch_wave sizes its grid).
int wave_grid(const sbp_ctx* ctx) {
  const int ty = wave_tile_height(8, wave_kind(ctx));
  const long long ntiles = ((ctx->nx + kWaveTX - 1) / kWaveTX) * ((ctx->ny + ty - 1) / ty);
  const int nsm = device_sm_count();
  return (int)(ntiles < nsm ? ntiles : nsm);
}

// One attempted step: six RHS evaluations with the stage combinations between
// them, then the candidate solution, the controller and the accept copy. The 2D
// wave problems fuse each combination into the stage kernel.
int enqueue_rk45_attempt(sbp_ctx* ctx) {
  const Rk45Buffers b = rk45_buffers(ctx);
  if (ctx->wave) {
    int rc;
    void* bufs[2] = {ctx->wa, ctx->wb};
    const WaveMaps* maps[2] = {&ctx->maps_wa, &ctx->maps_wb};
    for (int s = 1; s <= 6; s++) {
      void* in = s == 1 ? ctx->un : bufs[s % 2];           // s = 2: wa, 3: wb, 4: wa, ...
      const WaveMaps* m = s == 1 ? &ctx->maps_un : maps[s % 2];
      void* wout = s == 6 ? nullptr : bufs[(s + 1) % 2];  // s = 1: wa, 2: wb, ...
      if ((rc = launch_rkf_wave_stage(ctx, s, in, m, wout))) return rc;
    }
    CK(launch_rk45_control(b, wave_grid(ctx), ctx->rk_ctrl, ctx->stream));
    ctx->launches += 2;
    return SBP_OK;
  }
  for (int s = 0; s < 6; s++) {
    void* in = s == 0 ? ctx->un : ctx->wa;
    const WaveMaps* m = s == 0 ? &ctx->maps_un : &ctx->maps_wa;
    int rc = launch_stage<double>(ctx, ST_RHS, 0, 0.0, 0.0, in, m, ctx->rk_k[s], 1, ctx->rk_ctrl, kRkfC[s]);
    if (rc) return rc;
    if (s < 5) {
      CK(launch_rk45_combine(s + 1, b, ctx->rk_ctrl, ctx->stream));
      ctx->launches++;
    }
  }
  CK(launch_rk45_finish(b, ctx->rk_ctrl, ctx->stream));
  ctx->launches += 3;
  return SBP_OK;
}

constexpr int kRk45Chunk = 8;  // attempts per graph launch
// kernels per attempt: 6 fused stages + control + accept (2D wave), or
// 6 RHS + 5 combinations + final, control, accept
int rk45_launches_per_try(const sbp_ctx* ctx) { return ctx->wave ? 8 : 14; }

int rk45_chunk_graph(sbp_ctx* ctx) {
  if (ctx->rk_graph) return SBP_OK;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  const long long before = ctx->launches;
  int rc = SBP_OK;
  for (int a = 0; a < kRk45Chunk && rc == SBP_OK; a++) rc = enqueue_rk45_attempt(ctx);
  cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
  ctx->launches = before;  // captured, not yet run
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  CK(ce);
  cudaError_t ie = cudaGraphInstantiate(&ctx->rk_graph, g, 0);
  cudaGraphDestroy(g);
  CK(ie);
  return SBP_OK;
}

// First step under the landing rule of the controller (rk45.cu).
void rk45_first_step(double t0, double t_end, double dt0, double* h, int* fin) {
  const double hmax = t_end - t0;
  *h = dt0;
  *fin = 0;
  if (dt0 >= hmax) {
    *h = hmax;
    *fin = 1;
    return;
  }
  if (2.0 * dt0 > hmax) *h = 0.5 * hmax;
  if (1.01 * dt0 > hmax) {
    *h = hmax;
    *fin = 1;
  }
}

void release(sbp_ctx* ctx) {
  if (!ctx) return;
  drop_graphs(ctx);
  if (ctx->rk_graph) cudaGraphExecDestroy(ctx->rk_graph);
  for (int s = 0; s < 6; s++)
    if (ctx->rk_k[s]) cudaFree(ctx->rk_k[s]);
  if (ctx->rk_unew) cudaFree(ctx->rk_unew);
  if (ctx->rk_ctrl) cudaFree(ctx->rk_ctrl);
  void* bufs[] = {ctx->un, ctx->acc, ctx->wa, ctx->wb, ctx->comp, ctx->io, ctx->partial, ctx->red,
                  ctx->rinv, ctx->rho64, ctx->k64, ctx->err, ctx->sched, ctx->va, ctx->va64};
  // kmod lives inside the rinv allocation, vb and vb64 inside those of va and va64
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
}

}  // namespace

extern "C" {

int sbp_create(const sbp_desc* desc, sbp_ctx** out) {
  if (!desc || !out) return SBP_ERR_INVALID;
  *out = nullptr;
  sbp_ctx* ctx = new (std::nothrow) sbp_ctx();
  if (!ctx) return SBP_ERR_INVALID;
  ctx->d = *desc;
  const sbp_desc& d = ctx->d;
  auto bad = [&](const std::string& m) {
    g_create_error = m;
    delete ctx;
    return SBP_ERR_INVALID;
  };
  if (d.problem < SBP_WAVE_HOM_2D || d.problem > SBP_WAVE_3D) return bad("unknown problem");
  if (d.order != 2 && d.order != 4 && d.order != 6) return bad("order must be 2, 4 or 6");
  if (d.precision != SBP_FP64 && d.precision != SBP_FP32) return bad("unknown precision");
  if (d.bc != SBP_BC_REFERENCE && d.bc != SBP_BC_CHARACTERISTIC) return bad("unknown boundary treatment");
  ctx->two_d = is_2d(d.problem);
  ctx->three_d = d.problem == SBP_WAVE_3D;
  ctx->wave = is_wave(d.problem);
  ctx->dofs = dofs_of(d.problem);
  ctx->fp32 = d.precision == SBP_FP32;
  ctx->es = ctx->fp32 ? 4 : 8;
  ctx->nx = d.nx;
  ctx->ny = (ctx->two_d || ctx->three_d) ? d.ny : 1;
  ctx->nz = ctx->three_d ? d.nz : 1;
  const long long m = ops::min_points(d.order);
  if (ctx->nx < m || ((ctx->two_d || ctx->three_d) && ctx->ny < m) || (ctx->three_d && ctx->nz < m))
    return bad("grid smaller than the operator's minimum size");
  if (ctx->nx > (1LL << 30) || ctx->ny > (1LL << 30) || ctx->nz > (1LL << 20) ||
      (ctx->three_d && ctx->ny * ctx->nz > (1LL << 30)))
    return bad("grid too large");
  if (d.bc == SBP_BC_CHARACTERISTIC && !(d.problem == SBP_WAVE_HOM_2D || d.problem == SBP_WAVE_3D ||
                                          has_fields(d.problem)))
    return bad("characteristic boundary terms exist for the wave problems with rho, K fields only");
  if (d.problem == SBP_WAVE_MMS_2D && ctx->fp32) return bad("the manufactured-solution problem is FP64 only");
  if (has_fields(d.problem) && (!d.rho || !d.K)) return bad("rho and K are required");
  if (d.problem == SBP_WAVE_2BLOCK_2D && (ctx->ny % 2 || ctx->ny / 2 < m))
    return bad("two-block grids need an even ny with ny/2 at least the operator's minimum size");
  if (!(d.xr[0] > d.xl[0]) || ((ctx->two_d || ctx->three_d) && !(d.xr[1] > d.xl[1])) ||
      (ctx->three_d && !(d.xr2 > d.xl2)))
    return bad("empty domain");
  ctx->time_dependent = d.problem == SBP_WAVE_MMS_2D;
  ctx->hix = (ctx->nx - 1) / (d.xr[0] - d.xl[0]);
  ctx->hx = 1.0 / ctx->hix;
  if (ctx->two_d) {
    ctx->hiy = (ctx->ny - 1) / (d.xr[1] - d.xl[1]);
    if (d.problem == SBP_WAVE_2BLOCK_2D) {  // each block: ny/2 points over half the y extent
      ctx->ysplit = (int)(ctx->ny / 2);
      ctx->hiy = (ctx->ny / 2 - 1) / (0.5 * (d.xr[1] - d.xl[1]));
    }
    ctx->hy = 1.0 / ctx->hiy;
  }
  if (ctx->three_d) {
    ctx->hiy = (ctx->ny - 1) / (d.xr[1] - d.xl[1]);
    ctx->hy = 1.0 / ctx->hiy;
    ctx->hiz = (ctx->nz - 1) / (d.xr2 - d.xl2);
    ctx->hz = 1.0 / ctx->hiz;
  }
  ctx->pitch = (ctx->nx + 63) / 64 * 64;
  ctx->plane = ctx->pitch * ctx->ny * ctx->nz;
  ctx->npts = ctx->nx * ctx->ny * ctx->nz;
  ctx->nscalar = ctx->npts * ctx->dofs;

  if (cudaSetDevice(d.device) != cudaSuccess) return bad("cudaSetDevice failed");
  auto cuda_fail = [&](const char* what, cudaError_t e) {
    g_create_error = std::string(what) + ": " + cudaGetErrorString(e);
    release(ctx);
    delete ctx;
    return SBP_ERR_CUDA;
  };
  cudaError_t e;
  if (d.stream) {
    ctx->stream = (cudaStream_t)d.stream;
  } else {
    if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess)
      return cuda_fail("cudaStreamCreate", e);
    ctx->own_stream = true;
  }
  const size_t state_bytes = (size_t)ctx->dofs * ctx->plane * ctx->es;
  void** bufs[] = {&ctx->un, &ctx->acc, &ctx->wa, &ctx->wb};
  for (void** b : bufs) {
    if ((e = cudaMalloc(b, state_bytes)) != cudaSuccess) return cuda_fail("cudaMalloc(state)", e);
    cudaMemset(*b, 0, state_bytes);
  }
  if (ctx->fp32) {
    if ((e = cudaMalloc(&ctx->comp, state_bytes)) != cudaSuccess) return cuda_fail("cudaMalloc(comp)", e);
    cudaMemset(ctx->comp, 0, state_bytes);
  }
  if ((e = cudaMalloc((void**)&ctx->io, ctx->nscalar * sizeof(double))) != cudaSuccess)
    return cuda_fail("cudaMalloc(io)", e);
  if ((e = cudaMalloc((void**)&ctx->partial, 2 * kReduceBlocks * sizeof(double))) != cudaSuccess)
    return cuda_fail("cudaMalloc(partial)", e);
  if ((e = cudaMalloc((void**)&ctx->red, 4 * sizeof(double))) != cudaSuccess) return cuda_fail("cudaMalloc(red)", e);
  if ((e = cudaMalloc((void**)&ctx->err, sizeof(int))) != cudaSuccess) return cuda_fail("cudaMalloc(err)", e);
  cudaMemset(ctx->err, 0, sizeof(int));
  if ((e = cudaMalloc((void**)&ctx->sched, 2 * sizeof(int))) != cudaSuccess) return cuda_fail("cudaMalloc(sched)", e);
  cudaMemset(ctx->sched, 0, 2 * sizeof(int));

  if (has_fields(d.problem)) {
    const size_t np = (size_t)ctx->npts;
    double* rinv_h = new (std::nothrow) double[np];
    if (!rinv_h) return cuda_fail("host allocation", cudaErrorMemoryAllocation);
    for (size_t q = 0; q < np; q++) rinv_h[q] = 1.0 / d.rho[q];
    if ((e = cudaMalloc((void**)&ctx->rho64, np * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc((void**)&ctx->k64, np * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&ctx->rinv, 2 * ctx->plane * ctx->es)) != cudaSuccess) {
      delete[] rinv_h;
      return cuda_fail("cudaMalloc(coefficients)", e);
    }
    cudaMemset(ctx->rinv, 0, 2 * ctx->plane * ctx->es);
    ctx->kmod = static_cast<unsigned char*>(ctx->rinv) + ctx->plane * ctx->es;  // second plane
    cudaMemcpy(ctx->rho64, d.rho, np * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(ctx->k64, d.K, np * sizeof(double), cudaMemcpyHostToDevice);
    // pack 1/rho and K into padded planes of T via the AoS->SoA kernel (dofs = 1)
    double* tmp = nullptr;
    if ((e = cudaMalloc((void**)&tmp, np * sizeof(double))) != cudaSuccess) {
      delete[] rinv_h;
      return cuda_fail("cudaMalloc(tmp)", e);
    }
    cudaMemcpy(tmp, rinv_h, np * sizeof(double), cudaMemcpyHostToDevice);
    delete[] rinv_h;
    if (ctx->fp32) {
      launch_pack<float>(tmp, (float*)ctx->rinv, (int)ctx->nx, (int)ctx->ny, 1, ctx->pitch, ctx->plane, 0);
      launch_pack<float>(ctx->k64, (float*)ctx->kmod, (int)ctx->nx, (int)ctx->ny, 1, ctx->pitch, ctx->plane, 0);
    } else {
      launch_pack<double>(tmp, (double*)ctx->rinv, (int)ctx->nx, (int)ctx->ny, 1, ctx->pitch, ctx->plane, 0);
      launch_pack<double>(ctx->k64, (double*)ctx->kmod, (int)ctx->nx, (int)ctx->ny, 1, ctx->pitch, ctx->plane, 0);
    }
    e = cudaDeviceSynchronize();
    cudaFree(tmp);
    if (e != cudaSuccess) return cuda_fail("coefficient upload", e);
  }
  const bool adv = d.problem == SBP_ADVECTION_1D || d.problem == SBP_ADVECTION_2D;
  if (!adv && (d.a_field || d.b_field)) {
    g_create_error = "velocity fields are for the advection problems";
    release(ctx);
    delete ctx;
    return SBP_ERR_INVALID;
  }
  if (adv && (d.a_field || (ctx->two_d && d.b_field))) {
    // velocities at every point: FP64 copies for the SAT, planes of T for the interior
    const size_t np = (size_t)ctx->npts;
    double* host = new (std::nothrow) double[2 * np];
    if (!host) return cuda_fail("host allocation", cudaErrorMemoryAllocation);
    for (size_t q = 0; q < np; q++) {
      host[q] = d.a_field ? d.a_field[q] : d.a;
      host[np + q] = (ctx->two_d && d.b_field) ? d.b_field[q] : d.b;
    }
    const int nf = ctx->two_d ? 2 : 1;
    if ((e = cudaMalloc((void**)&ctx->va64, nf * np * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&ctx->va, nf * ctx->plane * ctx->es)) != cudaSuccess) {
      delete[] host;
      return cuda_fail("cudaMalloc(velocity fields)", e);
    }
    cudaMemset(ctx->va, 0, nf * ctx->plane * ctx->es);
    ctx->vb64 = ctx->va64 + (nf - 1) * np;  // 1D: vb is never read
    ctx->vb = static_cast<unsigned char*>(ctx->va) + (nf - 1) * ctx->plane * ctx->es;
    e = cudaMemcpy(ctx->va64, host, np * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nf == 2)
      e = cudaMemcpy(ctx->vb64, host + np, np * sizeof(double), cudaMemcpyHostToDevice);
    delete[] host;
    if (e != cudaSuccess) return cuda_fail("velocity upload", e);
    for (int f = 0; f < nf; f++) {
      const double* src = f == 0 ? ctx->va64 : ctx->vb64;
      void* dst = f == 0 ? ctx->va : ctx->vb;
      e = ctx->fp32 ? launch_pack<float>(src, (float*)dst, (int)ctx->nx, (int)ctx->ny, 1, ctx->pitch, ctx->plane, 0)
                    : launch_pack<double>(src, (double*)dst, (int)ctx->nx, (int)ctx->ny, 1, ctx->pitch, ctx->plane, 0);
      if (e != cudaSuccess) return cuda_fail("velocity packing", e);
    }
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return cuda_fail("velocity packing", e);
  }
  if (ctx->wave) {
    if (make_maps(ctx, ctx->un, ctx->maps_un) || make_maps(ctx, ctx->wa, ctx->maps_wa) ||
        make_maps(ctx, ctx->wb, ctx->maps_wb)) {
      g_create_error = ctx->msg;
      release(ctx);
      delete ctx;
      return SBP_ERR_CUDA;
    }
    // shared-memory opt-in of the stage kernels, done here (not under stream capture)
    e = ctx->fp32 ? configure_wave<float>(d.order, wave_kind(ctx)) : configure_wave<double>(d.order, wave_kind(ctx));
    if (e != cudaSuccess) return cuda_fail("configure stage kernels", e);
  }
  if (ctx->three_d) {
    e = ctx->fp32 ? configure_wave3d<float>(d.order) : configure_wave3d<double>(d.order);
    if (e != cudaSuccess) return cuda_fail("configure 3D stage kernels", e);
  }
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return cuda_fail("create", e);
  *out = ctx;
  return SBP_OK;
}

int sbp_destroy(sbp_ctx* ctx) {
  if (!ctx) return SBP_ERR_INVALID;
  cudaSetDevice(ctx->d.device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  release(ctx);
  delete ctx;
  return SBP_OK;
}

const char* sbp_last_error(const sbp_ctx* ctx) { return ctx ? ctx->msg.c_str() : g_create_error.c_str(); }

int sbp_dofs(const sbp_ctx* ctx) { return ctx ? ctx->dofs : SBP_ERR_INVALID; }

long long sbp_size(const sbp_ctx* ctx) { return ctx ? ctx->nscalar : SBP_ERR_INVALID; }

int sbp_rhs(sbp_ctx* ctx, double t, const double* src, double* dst, int where) {
  return rhs_impl(ctx, t, src, dst, where, 1);
}

int sbp_apply(sbp_ctx* ctx, double t, const double* src, double* dst, int where) {
  return rhs_impl(ctx, t, src, dst, where, 0);
}

long long sbp_rk4_nsteps(double t_end, double* dt) {
  if (!dt || !(*dt > 0) || !(t_end > 0)) return SBP_ERR_INVALID;
  const long long n = std::llround(t_end / *dt);
  if (n > 0 && std::fabs((double)n * *dt - t_end) > 1e-14) *dt = t_end / (double)n;
  return n;
}

int sbp_set_state(sbp_ctx* ctx, const double* v, int where) {
  if (!ctx) return SBP_ERR_INVALID;
  CK(cudaSetDevice(ctx->d.device));
  const double* dev = nullptr;
  int rc;
  if ((rc = stage_in(ctx, v, where, &dev))) return rc;
  if ((rc = pack_into(ctx, dev, ctx->un))) return rc;
  if (ctx->comp) CK(cudaMemsetAsync(ctx->comp, 0, (size_t)ctx->dofs * ctx->plane * ctx->es, ctx->stream));
  return SBP_OK;
}

int sbp_get_state(sbp_ctx* ctx, double* v, int where) {
  if (!ctx) return SBP_ERR_INVALID;
  CK(cudaSetDevice(ctx->d.device));
  int rc = unpack_to(ctx, ctx->un, v, where);
  if (rc) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  return SBP_OK;
}

int sbp_rk4_resident(sbp_ctx* ctx, double t0, double dt, long long nsteps) {
  if (!ctx) return SBP_ERR_INVALID;
  if (nsteps < 0 || !(dt > 0)) return fail(ctx, SBP_ERR_INVALID, "need dt > 0 and nsteps >= 0");
  CK(cudaSetDevice(ctx->d.device));
  return ctx->fp32 ? rk4_resident_t<float>(ctx, t0, dt, nsteps) : rk4_resident_t<double>(ctx, t0, dt, nsteps);
}

int sbp_synchronize(sbp_ctx* ctx) {
  if (!ctx) return SBP_ERR_INVALID;
  CK(cudaSetDevice(ctx->d.device));
  CK(cudaStreamSynchronize(ctx->stream));
  return check_device_errors(ctx);
}

int sbp_rk4(sbp_ctx* ctx, double t0, double dt, long long nsteps, double* v, int where) {
  int rc;
  if ((rc = sbp_set_state(ctx, v, where))) return rc;
  if ((rc = sbp_rk4_resident(ctx, t0, dt, nsteps))) return rc;
  if ((rc = sbp_get_state(ctx, v, where))) return rc;
  return check_device_errors(ctx);
}

int sbp_ts_rk4(sbp_ctx* ctx, double t_end, double dt, double* v, int where) {
  if (!ctx) return SBP_ERR_INVALID;
  double d = dt;
  const long long n = sbp_rk4_nsteps(t_end, &d);
  if (n < 0) return fail(ctx, SBP_ERR_INVALID, "need t_end > 0 and dt > 0");
  return sbp_rk4(ctx, 0.0, d, n, v, where);
}

int sbp_error_norms(sbp_ctx* ctx, const double* exact, int where, double* l2, double* linf) {
  if (!ctx || !l2 || !linf) return SBP_ERR_INVALID;
  CK(cudaSetDevice(ctx->d.device));
  const double* dev = nullptr;
  int rc;
  if ((rc = stage_in(ctx, exact, where, &dev))) return rc;
  if (ctx->fp32)
    CK(launch_error_norms<float>((const float*)ctx->un, dev, (int)ctx->nx, (int)(ctx->ny * ctx->nz), ctx->dofs,
                                 ctx->pitch,
                                 ctx->plane, ctx->partial, ctx->red, ctx->stream));
  else
    CK(launch_error_norms<double>((const double*)ctx->un, dev, (int)ctx->nx, (int)(ctx->ny * ctx->nz), ctx->dofs,
                                  ctx->pitch,
                                  ctx->plane, ctx->partial, ctx->red, ctx->stream));
  ctx->launches += 2;
  double h[2];
  CK(cudaMemcpyAsync(h, ctx->red, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const double hprod = (ctx->two_d || ctx->three_d) ? ctx->hx * ctx->hy * (ctx->three_d ? ctx->hz : 1.0) : ctx->hx;
  *l2 = std::sqrt(hprod) * std::sqrt(h[0]);
  *linf = h[1];
  return SBP_OK;
}

int sbp_hnorm(sbp_ctx* ctx, double* hn) {
  if (!ctx || !hn) return SBP_ERR_INVALID;
  CK(cudaSetDevice(ctx->d.device));
  if (ctx->fp32)
    CK(launch_hnorm<float>((const float*)ctx->un, (int)ctx->nx, (int)ctx->ny, ctx->dofs, ctx->pitch, ctx->plane,
                           ctx->d.order, ctx->hx, ctx->hy, ctx->ysplit, ctx->partial, ctx->red, ctx->stream,
                           (int)ctx->nz, ctx->hz));
  else
    CK(launch_hnorm<double>((const double*)ctx->un, (int)ctx->nx, (int)ctx->ny, ctx->dofs, ctx->pitch, ctx->plane,
                            ctx->d.order, ctx->hx, ctx->hy, ctx->ysplit, ctx->partial, ctx->red, ctx->stream,
                            (int)ctx->nz, ctx->hz));
  ctx->launches += 2;
  double h = 0;
  CK(cudaMemcpyAsync(&h, ctx->red, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *hn = std::sqrt(h);
  return SBP_OK;
}

void sbp_rk45_default_opts(sbp_rk45_opts* o) {
  if (!o) return;
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

int sbp_rk45_resident(sbp_ctx* ctx, double t0, double t_end, double dt0, const sbp_rk45_opts* opts,
                      sbp_rk45_stats* stats) {
  if (!ctx) return SBP_ERR_INVALID;
  if (ctx->fp32) return fail(ctx, SBP_ERR_UNSUPPORTED, "the adaptive RK45 integrator runs on FP64 contexts");
  if (!(dt0 > 0) || !(t_end >= t0)) return fail(ctx, SBP_ERR_INVALID, "need dt0 > 0 and t_end >= t0");
  sbp_rk45_opts o;
  sbp_rk45_default_opts(&o);
  if (opts) o = *opts;
  if (!(o.atol >= 0 && o.rtol >= 0 && o.atol + o.rtol > 0) || !(o.safety > 0) || !(o.reject_safety > 0) ||
      !(o.clip_lo > 0 && o.clip_hi >= o.clip_lo) || !(o.dt_min > 0 && o.dt_max >= o.dt_min) || o.max_steps < 1 ||
      o.max_reject < 1)
    return fail(ctx, SBP_ERR_INVALID, "invalid RK45 options");
  CK(cudaSetDevice(ctx->d.device));
  int rc;
  if ((rc = rk45_prepare(ctx))) return rc;
  if (ctx->rk_graph && (ctx->rk_atol != o.atol || ctx->rk_rtol != o.rtol)) {
    cudaGraphExecDestroy(ctx->rk_graph);
    ctx->rk_graph = nullptr;
  }
  ctx->rk_atol = o.atol;
  ctx->rk_rtol = o.rtol;
  if ((rc = rk45_chunk_graph(ctx))) return rc;
  Rk45Ctrl c;
  std::memset(&c, 0, sizeof(c));
  c.t = t0;
  c.t_end = t_end;
  c.atol = o.atol;
  c.rtol = o.rtol;
  c.safety = o.safety;
  c.reject_safety = o.reject_safety;
  c.clip_lo = o.clip_lo;
  c.clip_hi = o.clip_hi;
  c.dt_min = o.dt_min;
  c.dt_max = o.dt_max;
  c.max_steps = o.max_steps;
  c.max_reject = o.max_reject;
  c.n = (double)ctx->nscalar;  // every scalar of the state (nz slabs included)
  c.last_accepted = 1;
  c.status = RK45_OK;
  rk45_first_step(t0, t_end, std::fmin(dt0, o.dt_max), &c.h, &c.final_step);
  c.done = (t_end > t0) ? 0 : 1;
  CK(cudaMemcpyAsync(ctx->rk_ctrl, &c, sizeof(c), cudaMemcpyHostToDevice, ctx->stream));
  // every chunk advances the attempt count by kRk45Chunk until the controller stops
  const long long max_chunks = o.max_steps / kRk45Chunk + 2;
  for (long long chunk = 0; !c.done; chunk++) {
    if (chunk >= max_chunks) return fail(ctx, SBP_ERR_DEVICE, "the RK45 controller did not stop");
    CK(cudaGraphLaunch(ctx->rk_graph, ctx->stream));
    ctx->launches += (long long)kRk45Chunk * rk45_launches_per_try(ctx);
    CK(cudaMemcpyAsync(&c, ctx->rk_ctrl, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream));
    if ((rc = check_device_errors(ctx))) return rc;  // synchronizes the stream
  }
  if (stats) {
    stats->accepted = c.accepted;
    stats->rejected = c.rejected;
    stats->t = c.t;
    stats->dt_next = c.h;
    stats->wlte = c.wlte;
    stats->status = c.status;
  }
  if (c.status != RK45_OK) {
    static const char* why[] = {"", "the RK45 step limit was reached", "the RK45 error norm was not finite",
                                "too many RK45 rejections in a row"};
    return fail(ctx, SBP_ERR_DIVERGED, why[c.status]);
  }
  return SBP_OK;
}

int sbp_ts_rk45(sbp_ctx* ctx, double t_end, double dt, double* v, int where) {
  if (!ctx) return SBP_ERR_INVALID;
  int rc;
  if ((rc = sbp_set_state(ctx, v, where))) return rc;
  if ((rc = sbp_rk45_resident(ctx, 0.0, t_end, dt, nullptr, nullptr))) return rc;
  return sbp_get_state(ctx, v, where);
}

int sbp_set_wait_limit(sbp_ctx* ctx, long long ns) {
  if (!ctx) return SBP_ERR_INVALID;
  if (ns < 0 || ns > 60LL * 1000 * 1000 * 1000) return fail(ctx, SBP_ERR_INVALID, "wait limit must be in [0, 60 s]");
  CK(cudaSetDevice(ctx->d.device));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->wait_ns = (unsigned long long)ns;
  drop_graphs(ctx);  // captured launches carry the old limit
  if (ctx->rk_graph) {
    cudaGraphExecDestroy(ctx->rk_graph);
    ctx->rk_graph = nullptr;
  }
  return SBP_OK;
}

int sbp_test_drop_tile(sbp_ctx* ctx, long long tile) {
  if (!ctx) return SBP_ERR_INVALID;
  if (!ctx->wave) return fail(ctx, SBP_ERR_UNSUPPORTED, "the tile-drop test aid exists for the 2D wave kernels");
  const int ty = wave_tile_height((int)ctx->es, wave_kind(ctx));
  const long long ntiles = ((ctx->nx + kWaveTX - 1) / kWaveTX) * ((ctx->ny + ty - 1) / ty);
  if (tile < 0 || tile >= ntiles) return fail(ctx, SBP_ERR_INVALID, "tile index out of range");
  ctx->drop_tile = (int)(tile + 1);
  return SBP_OK;
}

int sbp_get_stream(const sbp_ctx* ctx, void** stream) {
  if (!ctx || !stream) return SBP_ERR_INVALID;
  *stream = (void*)ctx->stream;
  return SBP_OK;
}

long long sbp_launch_count(const sbp_ctx* ctx) { return ctx ? ctx->launches : SBP_ERR_INVALID; }

int sbp_probe_dfma_rate(int device, double* rate) {
  if (!rate) return SBP_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return SBP_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  double* out = nullptr;
  if (cudaMalloc((void**)&out, 2 * sizeof(double)) != cudaSuccess) return SBP_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  launch_dfma_probe(out, blocks, threads, 256, 0);  // warm-up
  cudaEventRecord(e0, 0);
  launch_dfma_probe(out, blocks, threads, iters, 0);
  cudaEventRecord(e1, 0);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess || ms <= 0) return SBP_ERR_CUDA;
  *rate = (double)blocks * threads * iters * 8.0 / (ms * 1e-3);
  return SBP_OK;
}

}  // extern "C"
