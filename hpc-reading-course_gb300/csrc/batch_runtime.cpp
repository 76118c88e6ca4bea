// batch_runtime.cpp -- the batched form behind include/sbpgpu.h (sbp_batch_*):
// many independent 2D wave (rho = 1, K = c^2) and 2D advection instances of
// uneven size and order, each with its own time step, advanced together.
//
// Device data: one pool per state buffer (u^n, acc, wa, wb, comp) holding
// every instance's SoA planes; an array of per-instance parameter blocks and
// (wave) tensor maps; per operator order, a tile list of (instance, tile)
// pairs. Each RK4 stage launches, per order group, one persistent wave kernel
// over its tile list and one advection kernel over its tiles. The step loop is
// captured into CUDA graphs of 100 steps, in which the six groups (order x
// problem kind), which share no data, are independent chains of launches: the
// device runs them side by side, so one group's tail and its memory-latency gaps
// are filled with another group's tiles.
//
// Autotuner: each group's kernel configuration (tile rows, compute warps, ring
// depth, CTAs per SM: the tables of wave_batch.cuh) is chosen by timing the
// group's middle stage on the batch itself; then the whole step is timed with
// those choices and with every group on each table entry, and the fastest kept.
// Choices are cached in a flat JSON file keyed by device, precision, problem
// kind, order and the group's size.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/sbpgpu.h"
#include "launch.h"
#include "sbp_ops.h"

using namespace sbp;

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

thread_local std::string g_batch_create_error;

struct Geo {
  bool wave;
  int order, dofs;
  long long nx, ny, pitch, plane;
  size_t off;  // byte offset of the instance's planes in each pool
};

}  // namespace

struct sbp_batch {
  int precision = SBP_FP64, device = 0;
  bool fp32 = false;
  size_t es = 8;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<sbp_instance> inst;
  std::vector<Geo> geo;
  size_t pool_bytes = 0, max_scalars = 0;
  void *un = nullptr, *acc = nullptr, *wa = nullptr, *wb = nullptr, *comp = nullptr;
  void* d_wave = nullptr;        // BatchWave<T>[n_wave]
  CUtensorMap* d_maps = nullptr; // kBatchMaps per wave instance
  void* d_line = nullptr;        // BatchLine<T>[n_line]
  CUtensorMap* d_maps_adv = nullptr;  // kAdvMaps per advection instance
  std::vector<int> wave_slot, line_slot;  // instance -> slot in d_wave / d_line (-1 if other kind)
  BatchTile* d_tiles_wave[3] = {nullptr, nullptr, nullptr};
  int n_tiles_wave[3] = {0, 0, 0};
  BatchTile* d_tiles_line[3] = {nullptr, nullptr, nullptr};
  int n_tiles_line[3] = {0, 0, 0};
  int cfg[6] = {0, 0, 0, 0, 0, 0};  // per group (2 * order index + kind): its configuration
  double* io = nullptr;
  int* err = nullptr;
  cudaStream_t gstream[6] = {};  // capture streams of the six groups' chains
  cudaEvent_t fork = nullptr, join[6] = {};
  std::map<long long, cudaGraphExec_t> graphs;
  long long launches = 0, points = 0;
  std::string msg;
};

namespace {

int bfail(sbp_batch* b, int code, const std::string& m) {
  if (b) b->msg = m;
  return code;
}

#define BCK(call)                                                                          \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return bfail(b, SBP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));   \
  } while (0)

int order_index(int order) { return order / 2 - 1; }

template <typename T>
void fill_taps(DirTaps<T>& t, int order, double scale) {
  const ops::Operator& op = ops::get(order);
  std::memset(&t, 0, sizeof(t));
  for (int s = 0; s < op.width; s++) t.taps[s] = (T)(scale * op.interior[s]);
  for (int r = 0; r < op.cls_sz; r++)
    for (int s = 0; s < op.cls_width; s++) t.cls[r][s] = (T)(scale * op.closure[r][s]);
}

void* at(void* pool, size_t off) { return pool ? static_cast<unsigned char*>(pool) + off : nullptr; }

// Encodes the tensor maps of instance i for tile height ty: the 12 of a wave
// instance (kBatchMaps) or the 6 of an advection instance (kAdvMaps).
int encode_instance_maps(sbp_batch* b, int i, int ty, CUtensorMap* out) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return bfail(b, SBP_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const Geo& g = b->geo[i];
  const int R = g.order / 2, hxa = 16 / (int)b->es;
  const int HX = (R + hxa - 1) / hxa * hxa, HY = R;
  const cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.dofs};
  const cuuint64_t strides[2] = {(cuuint64_t)(g.pitch * b->es), (cuuint64_t)(g.plane * b->es)};
  const cuuint32_t estr[3] = {1, 1, 1};
  const cuuint32_t boxP[3] = {(cuuint32_t)(kWaveTX + 2 * HX), (cuuint32_t)(ty + 2 * HY), 1};
  const cuuint32_t boxU[3] = {(cuuint32_t)(kWaveTX + 2 * HX), (cuuint32_t)ty, 1};
  const cuuint32_t boxV[3] = {(cuuint32_t)kWaveTX, (cuuint32_t)(ty + 2 * HY), 1};
  const cuuint32_t boxPt[3] = {(cuuint32_t)kWaveTX, (cuuint32_t)ty, (cuuint32_t)g.dofs};
  const CUtensorMapDataType dt = b->fp32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  void* inputs[3] = {at(b->un, g.off), at(b->wa, g.off), at(b->wb, g.off)};
  void* comp = b->comp ? at(b->comp, g.off) : at(b->acc, g.off);
  struct Req {
    void* base;
    const cuuint32_t* box;
  };
  const Req wave[kBatchMaps] = {{inputs[0], boxP}, {inputs[0], boxU}, {inputs[0], boxV}, {inputs[1], boxP},
                                {inputs[1], boxU}, {inputs[1], boxV}, {inputs[2], boxP}, {inputs[2], boxU},
                                {inputs[2], boxV}, {at(b->un, g.off), boxPt}, {at(b->acc, g.off), boxPt},
                                {comp, boxPt}};
  const Req adv[kAdvMaps] = {{inputs[0], boxP},          {inputs[1], boxP},           {inputs[2], boxP},
                             {at(b->un, g.off), boxPt}, {at(b->acc, g.off), boxPt}, {comp, boxPt}};
  const Req* reqs = g.wave ? wave : adv;
  const int n = g.wave ? kBatchMaps : kAdvMaps;
  for (int k = 0; k < n; k++)
    if (enc(&out[k], dt, 3, reqs[k].base, dims, strides, reqs[k].box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
        CUDA_SUCCESS)
      return bfail(b, SBP_ERR_CUDA, "cuTensorMapEncodeTiled failed for a batched instance");
  return SBP_OK;
}

// Group g = 2 * (order / 2 - 1) + kind (0 wave, 1 advection).
bool group_is_wave(int g) { return (g & 1) == 0; }
int group_order(int g) { return 2 * ((g >> 1) + 1); }
BatchTile*& group_tiles(sbp_batch* b, int g) { return (g & 1) ? b->d_tiles_line[g >> 1] : b->d_tiles_wave[g >> 1]; }
int& group_ntiles(sbp_batch* b, int g) { return (g & 1) ? b->n_tiles_line[g >> 1] : b->n_tiles_wave[g >> 1]; }
bool group_used(const sbp_batch* b, int g) {
  return (g & 1) ? b->n_tiles_line[g >> 1] > 0 : b->n_tiles_wave[g >> 1] > 0;
}
BatchCfg group_cfg(const sbp_batch* b, int g, int cfg) {
  return b->fp32 ? batch_cfg<float>(group_is_wave(g), cfg) : batch_cfg<double>(group_is_wave(g), cfg);
}

// (Re)builds the tensor maps and tile list of group g for configuration cfg.
int build_group(sbp_batch* b, int g, int cfg) {
  const int order = group_order(g);
  const bool wave = group_is_wave(g);
  const int ty = group_cfg(b, g, cfg).ty;
  std::vector<BatchTile> tiles;
  for (size_t i = 0; i < b->inst.size(); i++) {
    const Geo& geo = b->geo[i];
    if (geo.wave != wave || geo.order != order) continue;
    const int s = wave ? b->wave_slot[i] : b->line_slot[i];
    for (long long j0 = 0; j0 < geo.ny; j0 += ty)
      for (long long i0 = 0; i0 < geo.nx; i0 += kWaveTX) tiles.push_back(BatchTile{s, (int)i0, (int)j0, 0});
    CUtensorMap m[kBatchMaps];
    int rc = encode_instance_maps(b, (int)i, ty, m);
    if (rc) return rc;
    CUtensorMap* dst = wave ? b->d_maps + (size_t)s * kBatchMaps : b->d_maps_adv + (size_t)s * kAdvMaps;
    BCK(cudaMemcpyAsync(dst, m, (wave ? kBatchMaps : kAdvMaps) * sizeof(CUtensorMap), cudaMemcpyHostToDevice,
                        b->stream));
  }
  BatchTile*& d = group_tiles(b, g);
  if (d) cudaFree(d);
  d = nullptr;
  group_ntiles(b, g) = (int)tiles.size();
  if (!tiles.empty()) {
    BCK(cudaMalloc((void**)&d, tiles.size() * sizeof(BatchTile)));
    BCK(cudaMemcpyAsync(d, tiles.data(), tiles.size() * sizeof(BatchTile), cudaMemcpyHostToDevice, b->stream));
    BCK(b->fp32 ? configure_batch<float>(order, wave, cfg) : configure_batch<double>(order, wave, cfg));
  }
  b->cfg[g] = cfg;
  BCK(cudaStreamSynchronize(b->stream));
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
  return SBP_OK;
}

template <typename T>
int fill_params(sbp_batch* b) {
  std::vector<BatchWave<T>> waves;
  std::vector<BatchLine<T>> lines;
  for (size_t i = 0; i < b->inst.size(); i++) {
    const sbp_instance& d = b->inst[i];
    const Geo& g = b->geo[i];
    const double hix = (g.nx - 1) / (d.xr[0] - d.xl[0]), hiy = (g.ny - 1) / (d.xr[1] - d.xl[1]);
    const double hi0 = ops::get(d.order).hinv0;
    if (g.wave) {
      BatchWave<T> w;
      std::memset(&w, 0, sizeof(w));
      WaveParams<T>& p = w.prm;
      p.nx = (int)g.nx;
      p.ny = (int)g.ny;
      p.pitch = g.pitch;
      p.plane = g.plane;
      p.un = (T*)at(b->un, g.off);
      p.acc = (T*)at(b->acc, g.off);
      p.comp = (T*)at(b->comp, g.off);
      fill_taps<T>(p.dx, d.order, -hix);
      fill_taps<T>(p.dy, d.order, -hiy);
      p.bwx = hix * hi0;
      p.bwy = hiy * hi0;
      p.kconst = (T)(d.c * d.c);
      p.kz = p.kc = std::sqrt((double)p.kconst);  // sqrt(rho K) = sqrt(K / rho) with rho = 1, rounded alike
      p.dt = d.dt;
      p.bc = d.bc == SBP_BC_CHARACTERISTIC ? BC_CHARACTERISTIC : BC_FREE_SURFACE;
      p.err = b->err;
      w.wa = (T*)at(b->wa, g.off);
      w.wb = (T*)at(b->wb, g.off);
      batch_rk4_coefficients<T>(d.dt, w.c_acc, w.c_w);
      // the fixed-point entries' scales: sigma = -hi/den per direction, the p equation's
      // times K; each stage's coefficients times each component's scale
      const double den = d.order == 2 ? 2.0 : (d.order == 4 ? 12.0 : 60.0);
      p.fx_sig[0] = -hix / den;
      p.fx_sig[1] = -hiy / den;
      p.fx_isig[0] = -den / hix;
      p.fx_isig[1] = -den / hiy;
      p.fx_rho = hiy / hix;
      p.fx_square = hix == hiy ? 1 : 0;
      p.fx_sigp = p.fx_sig[0] * (double)p.kconst;
      const double sg[3] = {p.fx_sig[0], p.fx_sig[1], p.fx_sigp};
      for (int rk = 0; rk < 4; rk++)
        for (int c = 0; c < 3; c++) {
          w.fxa[rk][c] = (double)w.c_acc[rk] * sg[c];
          w.fxw[rk][c] = (double)w.c_w[rk] * sg[c];
        }
      waves.push_back(w);
    } else {
      BatchLine<T> l;
      std::memset(&l, 0, sizeof(l));
      LineParams<T>& p = l.prm;
      p.nx = (int)g.nx;
      p.ny = (int)g.ny;
      p.pitch = g.pitch;
      p.plane = g.plane;
      p.un = (T*)at(b->un, g.off);
      p.acc = (T*)at(b->acc, g.off);
      p.comp = (T*)at(b->comp, g.off);
      fill_taps<T>(p.dx, d.order, -d.a * hix);
      fill_taps<T>(p.dy, d.order, -d.b * hiy);
      p.sat[0] = 0.5 * (-0.5 * (d.a + std::fabs(d.a))) * (hix * hi0);
      p.sat[1] = 0.5 * (-0.5 * (d.b + std::fabs(d.b))) * (hiy * hi0);
      p.sat[2] = 0.5 * (0.5 * (d.a - std::fabs(d.a))) * (hix * hi0);
      p.sat[3] = 0.5 * (0.5 * (d.b - std::fabs(d.b))) * (hiy * hi0);
      p.bc = 1;
      p.compensated = b->fp32 ? 1 : 0;
      p.err = b->err;
      l.wa = (T*)at(b->wa, g.off);
      l.wb = (T*)at(b->wb, g.off);
      l.dt = d.dt;
      batch_rk4_coefficients<T>(d.dt, l.c_acc, l.c_w);
      lines.push_back(l);
    }
  }
  if (!waves.empty()) {
    BCK(cudaMalloc(&b->d_wave, waves.size() * sizeof(BatchWave<T>)));
    BCK(cudaMemcpy(b->d_wave, waves.data(), waves.size() * sizeof(BatchWave<T>), cudaMemcpyHostToDevice));
    BCK(cudaMalloc((void**)&b->d_maps, waves.size() * kBatchMaps * sizeof(CUtensorMap)));
  }
  if (!lines.empty()) {
    BCK(cudaMalloc(&b->d_line, lines.size() * sizeof(BatchLine<T>)));
    BCK(cudaMemcpy(b->d_line, lines.data(), lines.size() * sizeof(BatchLine<T>), cudaMemcpyHostToDevice));
    BCK(cudaMalloc((void**)&b->d_maps_adv, lines.size() * kAdvMaps * sizeof(CUtensorMap)));
  }
  for (int g = 0; g < 6; g++)
    if (int rc = build_group(b, g, 0)) return rc;
  return SBP_OK;
}

// One stage of group g with configuration cfg on stream s.
template <typename T>
cudaError_t launch_group_stage_cfg(sbp_batch* b, int g, int cfg, int stage, int rk, cudaStream_t s) {
  const bool wave = group_is_wave(g);
  return launch_batch<T>(group_order(g), wave, stage, cfg, wave ? b->d_wave : b->d_line,
                         wave ? b->d_maps : b->d_maps_adv, group_tiles(b, g), group_ntiles(b, g), rk, b->err, s);
}

template <typename T>
int launch_group_stage(sbp_batch* b, int g, int stage, int rk, cudaStream_t s) {
  BCK(launch_group_stage_cfg<T>(b, g, b->cfg[g], stage, rk, s));
  b->launches++;
  return SBP_OK;
}

// `steps` RK4 steps of group g on stream s.
template <typename T>
int enqueue_group(sbp_batch* b, int g, long long steps, cudaStream_t s) {
  static const int kStages[4][2] = {{ST_FIRST, 1}, {ST_MID, 2}, {ST_MID, 3}, {ST_LAST, 4}};
  for (long long n = 0; n < steps; n++)
    for (const auto& st : kStages)
      if (int rc = launch_group_stage<T>(b, g, st[0], st[1], s)) return rc;
  return SBP_OK;
}

// The chunk's launches while b->stream is capturing: each used group's chain on its
// own stream, forked from and joined back into b->stream.
template <typename T>
int enqueue_chunk(sbp_batch* b, long long steps) {
  BCK(cudaEventRecord(b->fork, b->stream));
  for (int g = 0; g < 6; g++) {
    if (!group_used(b, g)) continue;
    BCK(cudaStreamWaitEvent(b->gstream[g], b->fork, 0));
    if (int rc = enqueue_group<T>(b, g, steps, b->gstream[g])) return rc;
    BCK(cudaEventRecord(b->join[g], b->gstream[g]));
    BCK(cudaStreamWaitEvent(b->stream, b->join[g], 0));
  }
  return SBP_OK;
}

long long kernels_per_step(const sbp_batch* b) {
  long long n = 0;
  for (int oi = 0; oi < 3; oi++) n += (b->n_tiles_wave[oi] ? 1 : 0) + (b->n_tiles_line[oi] ? 1 : 0);
  return 4 * n;
}

template <typename T>
int run_chunk(sbp_batch* b, long long steps) {
  auto it = b->graphs.find(steps);
  if (it == b->graphs.end()) {
    cudaGraph_t g = nullptr;
    BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = b->launches;
    const int rc = enqueue_chunk<T>(b, steps);
    cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    b->launches = before;
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    BCK(ce);
    cudaGraphExec_t ex = nullptr;
    cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    BCK(ie);
    it = b->graphs.emplace(steps, ex).first;
  }
  BCK(cudaGraphLaunch(it->second, b->stream));
  b->launches += kernels_per_step(b) * steps;
  return SBP_OK;
}

// Among the per-group choices and the four uniform assignments (every group on entry e),
// keeps the one whose whole step -- all groups, their chains side by side -- is fastest:
// a group timed alone does not see how the groups share the device. The states (u^n, and
// comp in FP32) are saved before the trial steps and restored after them.
template <typename T>
int whole_step_choice(sbp_batch* b) {
  constexpr long long kSteps = 5;
  constexpr int NC = kBatchCfgs + 1;
  int cand[NC][6];
  for (int g = 0; g < 6; g++) {
    cand[0][g] = b->cfg[g];
    for (int e = 0; e < kBatchCfgs; e++) cand[e + 1][g] = e;
  }
  struct Scratch {
    void* un = nullptr;
    void* comp = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~Scratch() {
      if (un) cudaFree(un);
      if (comp) cudaFree(comp);
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
    }
  } sc;
  BCK(cudaEventCreate(&sc.e0));
  BCK(cudaEventCreate(&sc.e1));
  BCK(cudaMalloc(&sc.un, b->pool_bytes));
  if (b->comp) BCK(cudaMalloc(&sc.comp, b->pool_bytes));
  BCK(cudaMemcpyAsync(sc.un, b->un, b->pool_bytes, cudaMemcpyDeviceToDevice, b->stream));
  if (b->comp) BCK(cudaMemcpyAsync(sc.comp, b->comp, b->pool_bytes, cudaMemcpyDeviceToDevice, b->stream));
  // from here on every path restores the states
  const long long launches = b->launches;
  float best_ms = 1e30f;
  int best = 0, rc = SBP_OK;
  auto cuda = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && rc == SBP_OK) rc = bfail(b, SBP_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return rc == SBP_OK;
  };
  for (int c = 0; c < NC && rc == SBP_OK; c++) {
    for (int g = 0; g < 6 && rc == SBP_OK; g++)
      if (group_used(b, g) && b->cfg[g] != cand[c][g]) rc = build_group(b, g, cand[c][g]);
    if (rc || (rc = run_chunk<T>(b, kSteps))) break;  // captures this assignment's graph
    if (!cuda(cudaEventRecord(sc.e0, b->stream), "cudaEventRecord")) break;
    if ((rc = run_chunk<T>(b, kSteps))) break;
    float ms = 0;
    if (!cuda(cudaEventRecord(sc.e1, b->stream), "cudaEventRecord") ||
        !cuda(cudaEventSynchronize(sc.e1), "trial steps") || !cuda(cudaEventElapsedTime(&ms, sc.e0, sc.e1), "timing"))
      break;
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  }
  for (int g = 0; g < 6 && rc == SBP_OK; g++)
    if (group_used(b, g) && b->cfg[g] != cand[best][g]) rc = build_group(b, g, cand[best][g]);
  cuda(cudaMemcpyAsync(b->un, sc.un, b->pool_bytes, cudaMemcpyDeviceToDevice, b->stream), "state restore");
  if (b->comp)
    cuda(cudaMemcpyAsync(b->comp, sc.comp, b->pool_bytes, cudaMemcpyDeviceToDevice, b->stream), "state restore");
  cuda(cudaStreamSynchronize(b->stream), "state restore");
  b->launches = launches;
  return rc;
}

// ---- tiny flat JSON cache {"key": int, ...}
std::map<std::string, int> read_cache(const char* path) {
  std::map<std::string, int> m;
  if (!path) return m;
  FILE* f = std::fopen(path, "rb");
  if (!f) return m;
  std::string s;
  char buf[4096];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, n);
  std::fclose(f);
  size_t p = 0;
  while ((p = s.find('"', p)) != std::string::npos) {
    const size_t q = s.find('"', p + 1);
    if (q == std::string::npos) break;
    const std::string key = s.substr(p + 1, q - p - 1);
    const size_t c = s.find(':', q);
    if (c == std::string::npos) break;
    m[key] = std::atoi(s.c_str() + c + 1);
    p = s.find_first_of(",}", c);
    if (p == std::string::npos) break;
  }
  return m;
}

void write_cache(const char* path, const std::map<std::string, int>& m) {
  if (!path) return;
  FILE* f = std::fopen(path, "wb");
  if (!f) return;
  std::fputs("{", f);
  bool first = true;
  for (const auto& kv : m) {
    std::fprintf(f, "%s\n  \"%s\": %d", first ? "" : ",", kv.first.c_str(), kv.second);
    first = false;
  }
  std::fputs("\n}\n", f);
  std::fclose(f);
}

void release(sbp_batch* b) {
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
  void* bufs[] = {b->un, b->acc, b->wa, b->wb, b->comp, b->d_wave, b->d_maps, b->d_line, b->d_maps_adv, b->io, b->err};
  for (void* p : bufs)
    if (p) cudaFree(p);
  for (int oi = 0; oi < 3; oi++) {
    if (b->d_tiles_wave[oi]) cudaFree(b->d_tiles_wave[oi]);
    if (b->d_tiles_line[oi]) cudaFree(b->d_tiles_line[oi]);
  }
  for (int g = 0; g < 6; g++) {
    if (b->gstream[g]) cudaStreamDestroy(b->gstream[g]);
    if (b->join[g]) cudaEventDestroy(b->join[g]);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
}

}  // namespace

extern "C" {

int sbp_batch_create(const sbp_instance* list, int count, int precision, int device, void* stream, sbp_batch** out) {
  if (!list || count <= 0 || !out) {
    g_batch_create_error = "need a non-empty instance list and an output pointer";
    return SBP_ERR_INVALID;
  }
  *out = nullptr;
  if (precision != SBP_FP64 && precision != SBP_FP32) {
    g_batch_create_error = "unknown precision";
    return SBP_ERR_INVALID;
  }
  sbp_batch* b = new (std::nothrow) sbp_batch();
  if (!b) return SBP_ERR_INVALID;
  b->precision = precision;
  b->fp32 = precision == SBP_FP32;
  b->es = b->fp32 ? 4 : 8;
  b->device = device;
  b->inst.assign(list, list + count);
  size_t off = 0;
  int nw = 0, nl = 0;
  for (int i = 0; i < count; i++) {
    const sbp_instance& d = list[i];
    const bool wave = d.problem == SBP_WAVE_HOM_2D;
    std::string bad;
    if (!wave && d.problem != SBP_ADVECTION_2D) bad = "instances must be SBP_WAVE_HOM_2D or SBP_ADVECTION_2D";
    else if (d.order != 2 && d.order != 4 && d.order != 6) bad = "order must be 2, 4 or 6";
    else if (d.nx < ops::min_points(d.order) || d.ny < ops::min_points(d.order) || d.nx > (1 << 20) || d.ny > (1 << 20))
      bad = "grid outside [operator minimum, 2^20] points per direction";
    else if (!(d.xr[0] > d.xl[0]) || !(d.xr[1] > d.xl[1])) bad = "empty domain";
    else if (!(d.dt > 0)) bad = "dt must be positive";
    else if (wave && !(d.c > 0)) bad = "wave speed must be positive";
    else if (wave && d.bc != SBP_BC_REFERENCE && d.bc != SBP_BC_CHARACTERISTIC) bad = "unknown boundary treatment";
    if (!bad.empty()) {
      g_batch_create_error = "instance " + std::to_string(i) + ": " + bad;
      delete b;
      return SBP_ERR_INVALID;
    }
    Geo g;
    g.wave = wave;
    g.order = d.order;
    g.dofs = wave ? 3 : 1;
    g.nx = d.nx;
    g.ny = d.ny;
    g.pitch = (d.nx + 63) / 64 * 64;
    g.plane = g.pitch * d.ny;
    g.off = off;
    off += ((size_t)g.dofs * g.plane * b->es + 255) / 256 * 256;
    b->geo.push_back(g);
    b->wave_slot.push_back(wave ? nw++ : -1);
    b->line_slot.push_back(wave ? -1 : nl++);
    b->points += d.nx * d.ny;
    b->max_scalars = std::max(b->max_scalars, (size_t)(g.dofs * d.nx * d.ny));
  }
  b->pool_bytes = off;
  auto cuda_fail = [&](const char* what, cudaError_t e) {
    g_batch_create_error = std::string(what) + ": " + cudaGetErrorString(e);
    release(b);
    delete b;
    return SBP_ERR_CUDA;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(device)) != cudaSuccess) return cuda_fail("cudaSetDevice", e);
  if (stream) {
    b->stream = (cudaStream_t)stream;
  } else {
    if ((e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess)
      return cuda_fail("cudaStreamCreate", e);
    b->own_stream = true;
  }
  for (int g = 0; g < 6; g++) {
    if ((e = cudaStreamCreateWithFlags(&b->gstream[g], cudaStreamNonBlocking)) != cudaSuccess)
      return cuda_fail("cudaStreamCreate(group)", e);
    if ((e = cudaEventCreateWithFlags(&b->join[g], cudaEventDisableTiming)) != cudaSuccess)
      return cuda_fail("cudaEventCreate", e);
  }
  if ((e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess)
    return cuda_fail("cudaEventCreate", e);
  void** pools[] = {&b->un, &b->acc, &b->wa, &b->wb};
  for (void** p : pools) {
    if ((e = cudaMalloc(p, b->pool_bytes)) != cudaSuccess) return cuda_fail("cudaMalloc(pool)", e);
    cudaMemset(*p, 0, b->pool_bytes);
  }
  if (b->fp32) {
    if ((e = cudaMalloc(&b->comp, b->pool_bytes)) != cudaSuccess) return cuda_fail("cudaMalloc(comp)", e);
    cudaMemset(b->comp, 0, b->pool_bytes);
  }
  if ((e = cudaMalloc((void**)&b->io, b->max_scalars * sizeof(double))) != cudaSuccess)
    return cuda_fail("cudaMalloc(io)", e);
  if ((e = cudaMalloc((void**)&b->err, sizeof(int))) != cudaSuccess) return cuda_fail("cudaMalloc(err)", e);
  cudaMemset(b->err, 0, sizeof(int));
  const int rc = b->fp32 ? fill_params<float>(b) : fill_params<double>(b);
  if (rc) {
    g_batch_create_error = b->msg;
    release(b);
    delete b;
    return rc;
  }
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return cuda_fail("batch set-up", e);
  *out = b;
  return SBP_OK;
}

int sbp_batch_destroy(sbp_batch* b) {
  if (!b) return SBP_ERR_INVALID;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  release(b);
  delete b;
  return SBP_OK;
}

const char* sbp_batch_last_error(const sbp_batch* b) { return b ? b->msg.c_str() : g_batch_create_error.c_str(); }

int sbp_batch_set_state(sbp_batch* b, int index, const double* v, int where) {
  if (!b || !v || index < 0 || index >= (int)b->inst.size()) return SBP_ERR_INVALID;
  BCK(cudaSetDevice(b->device));
  const Geo& g = b->geo[index];
  const size_t n = (size_t)g.dofs * g.nx * g.ny;
  const double* src = v;
  if (where == SBP_HOST) {
    BCK(cudaMemcpyAsync(b->io, v, n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    src = b->io;
  } else if (where != SBP_DEVICE) {
    return bfail(b, SBP_ERR_INVALID, "where must be SBP_HOST or SBP_DEVICE");
  }
  if (b->fp32) {
    BCK(launch_pack<float>(src, (float*)at(b->un, g.off), (int)g.nx, (int)g.ny, g.dofs, g.pitch, g.plane, b->stream));
    BCK(cudaMemsetAsync(at(b->comp, g.off), 0, (size_t)g.dofs * g.plane * b->es, b->stream));
  } else {
    BCK(launch_pack<double>(src, (double*)at(b->un, g.off), (int)g.nx, (int)g.ny, g.dofs, g.pitch, g.plane,
                            b->stream));
  }
  b->launches++;
  BCK(cudaStreamSynchronize(b->stream));
  return SBP_OK;
}

int sbp_batch_get_state(sbp_batch* b, int index, double* v, int where) {
  if (!b || !v || index < 0 || index >= (int)b->inst.size()) return SBP_ERR_INVALID;
  if (where != SBP_HOST && where != SBP_DEVICE) return bfail(b, SBP_ERR_INVALID, "where must be SBP_HOST or SBP_DEVICE");
  BCK(cudaSetDevice(b->device));
  const Geo& g = b->geo[index];
  const size_t n = (size_t)g.dofs * g.nx * g.ny;
  double* dst = (where == SBP_DEVICE) ? v : b->io;
  if (b->fp32)
    BCK(launch_unpack<float>((const float*)at(b->un, g.off), dst, (int)g.nx, (int)g.ny, g.dofs, g.pitch, g.plane,
                             b->stream));
  else
    BCK(launch_unpack<double>((const double*)at(b->un, g.off), dst, (int)g.nx, (int)g.ny, g.dofs, g.pitch, g.plane,
                              b->stream));
  b->launches++;
  if (where != SBP_DEVICE)
    BCK(cudaMemcpyAsync(v, b->io, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return SBP_OK;
}

int sbp_batch_rk4_resident(sbp_batch* b, long long nsteps) {
  if (!b || nsteps < 0) return SBP_ERR_INVALID;
  BCK(cudaSetDevice(b->device));
  const long long chunk = 100;
  long long left = nsteps;
  while (left > 0) {
    const long long s = left >= chunk ? chunk : left;
    const int rc = b->fp32 ? run_chunk<float>(b, s) : run_chunk<double>(b, s);
    if (rc) return rc;
    left -= s;
  }
  return SBP_OK;
}

int sbp_batch_synchronize(sbp_batch* b) {
  if (!b) return SBP_ERR_INVALID;
  BCK(cudaSetDevice(b->device));
  BCK(cudaStreamSynchronize(b->stream));
  int h = 0;
  BCK(cudaMemcpy(&h, b->err, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    cudaMemset(b->err, 0, sizeof(int));
    return bfail(b, SBP_ERR_DEVICE, "a TMA tile wait timed out in a batched stage kernel");
  }
  return SBP_OK;
}

int sbp_batch_autotune(sbp_batch* b, const char* cache_path) {
  if (!b) return SBP_ERR_INVALID;
  BCK(cudaSetDevice(b->device));
  cudaDeviceProp prop;
  BCK(cudaGetDeviceProperties(&prop, b->device));
  std::map<std::string, int> cache = read_cache(cache_path);
  bool dirty = false;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int rc = SBP_OK;
  std::vector<std::pair<int, std::string>> keys;  // (group, cache key) of the groups in the batch
  bool timed = false;                              // a group missed the cache: choices to confirm
  for (int g = 0; g < 6 && rc == SBP_OK; g++) {
    const int order = group_order(g);
    const bool wave = group_is_wave(g);
    long long pts = 0;
    for (size_t i = 0; i < b->inst.size(); i++)
      if (b->geo[i].wave == wave && b->geo[i].order == order) pts += b->geo[i].nx * b->geo[i].ny;
    if (!pts) continue;
    // key: device, precision, kind, order, group size rounded to 2 significant digits
    const double mag = std::pow(10.0, std::floor(std::log10((double)pts)) - 1);
    const long long bucket = (long long)(std::round(pts / mag) * mag);
    const std::string key = std::string(prop.name) + "|" + (b->fp32 ? "fp32" : "fp64") + "|" +
                            (wave ? "wave" : "advection") + "|order" + std::to_string(order) + "|points" +
                            std::to_string(bucket) + "|cfg";
    keys.emplace_back(g, key);
    auto hit = cache.find(key);
    if (hit != cache.end() && hit->second >= 0 && hit->second < kBatchCfgs) {
      if (hit->second != b->cfg[g]) rc = build_group(b, g, hit->second);
      continue;
    }
    timed = true;
    float best_ms = 1e30f;
    int best = 0;
    for (int c = 0; c < kBatchCfgs && rc == SBP_OK; c++) {
      if ((rc = build_group(b, g, c))) break;
      // time the middle stage (it writes only the accumulator and a stage buffer): one
      // untimed launch, then three
      float ms = 0;
      for (int rep = 0; rep < 4 && rc == SBP_OK; rep++) {
        if (rep == 1) cudaEventRecord(e0, b->stream);
        if ((b->fp32 ? launch_group_stage_cfg<float>(b, g, c, ST_MID, 2, b->stream)
                     : launch_group_stage_cfg<double>(b, g, c, ST_MID, 2, b->stream)) != cudaSuccess)
          rc = bfail(b, SBP_ERR_CUDA, "autotune launch failed");
      }
      cudaEventRecord(e1, b->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) rc = bfail(b, SBP_ERR_CUDA, "autotune launch failed");
      cudaEventElapsedTime(&ms, e0, e1);
      if (rc == SBP_OK && ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
    if (rc == SBP_OK && best != b->cfg[g]) rc = build_group(b, g, best);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == SBP_OK && timed) rc = b->fp32 ? whole_step_choice<float>(b) : whole_step_choice<double>(b);
  if (rc) return bfail(b, rc, b->msg.empty() ? "autotune failed" : b->msg);
  if (timed) {
    for (const auto& k : keys) cache[k.second] = b->cfg[k.first];
    dirty = true;
  }
  if (dirty) write_cache(cache_path, cache);
  return sbp_batch_synchronize(b);
}

int sbp_batch_tile_height(const sbp_batch* b, int order) {
  if (!b || (order != 2 && order != 4 && order != 6)) return SBP_ERR_INVALID;
  const int g = 2 * order_index(order);
  return group_used(b, g) ? group_cfg(b, g, b->cfg[g]).ty : 0;
}

int sbp_batch_select_config(sbp_batch* b, int order, int problem, int index) {
  if (!b || (order != 2 && order != 4 && order != 6) ||
      (problem != SBP_WAVE_HOM_2D && problem != SBP_ADVECTION_2D) || index < 0 || index >= kBatchCfgs)
    return SBP_ERR_INVALID;
  BCK(cudaSetDevice(b->device));
  const int g = 2 * order_index(order) + (problem == SBP_ADVECTION_2D ? 1 : 0);
  return index == b->cfg[g] ? SBP_OK : build_group(b, g, index);
}

int sbp_batch_kernel_config(const sbp_batch* b, int order, int problem, int* cfg) {
  if (!b || !cfg || (order != 2 && order != 4 && order != 6) ||
      (problem != SBP_WAVE_HOM_2D && problem != SBP_ADVECTION_2D))
    return SBP_ERR_INVALID;
  const int g = 2 * order_index(order) + (problem == SBP_ADVECTION_2D ? 1 : 0);
  if (!group_used(b, g)) {
    cfg[0] = cfg[1] = cfg[2] = cfg[3] = cfg[4] = 0;
    return SBP_OK;
  }
  const BatchCfg c = group_cfg(b, g, b->cfg[g]);
  cfg[0] = c.ty;
  cfg[1] = c.warps;
  cfg[2] = c.nst;
  cfg[3] = c.ctas;
  cfg[4] = c.conv;
  return SBP_OK;
}

int sbp_batch_get_stream(const sbp_batch* b, void** stream) {
  if (!b || !stream) return SBP_ERR_INVALID;
  *stream = (void*)b->stream;
  return SBP_OK;
}

long long sbp_batch_points(const sbp_batch* b) { return b ? b->points : SBP_ERR_INVALID; }

long long sbp_batch_launch_count(const sbp_batch* b) { return b ? b->launches : SBP_ERR_INVALID; }

}  // extern "C"
