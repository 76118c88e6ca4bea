// decomp.cu -- the 2D wave system (rho = K = 1, FP64) on a P x Q decomposition of
// one grid, on one GPU: each subdomain holds its own SoA state with R ghost lines
// on each side, and one launch per RK4 stage evaluates the RHS and the stage
// update of all subdomains while refreshing the ghosts the next stage reads. It is
// the reference's decomposed path -- rhs_local / rhs_all over a DMDA block grid
// (code/include/partitioned_rhs/rhs.h:97-181, 183-360) with the VecScatter ghost
// update of code/src/scatter/scatter_ctx.cpp:149-211 -- with the halo exchange on
// the device, the step towards one subdomain per GPU.
//
// The stage kernel is the single grid's fixed-point FP64 kernel with converter
// warps (wave2d_fixed.cuh, wave_fixed_kernel<ORD, STAGE, true>) over the
// subdomains' tile list: its producer loads each tile's p/u/v boxes, ghosts
// included, with TMA maps of the tile's subdomain, and the compute warps take the
// central stencil across internal edges from the ghosts and closure rows and SAT
// terms only at the physical boundary (global indices), so a decomposed run
// matches the single grid to rounding. A subdomain's arrays keep ghost_x(order)
// ghost columns (R rounded up to an even count: TMA x coordinates must be 16-byte
// aligned) and R ghost rows. In the RK4 loop the exchange is fused into the
// stages: the kernel's exchange warp copies each finished tile's points within R
// of an internal edge into the neighbour's mirroring ghost line, so the exchange
// overlaps the stage's computation and costs no launch (the reference overlaps
// its VecScatter with rhs_local, code/demo/wave_hom/wave_eq_hom_sim.cpp:258-261).
// The halo kernel remains for states set from outside (before an RHS, at the
// start of a run of steps).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "../../include/sbpgpu.h"
#include "launch.h"
#include "sbp_ops.h"

namespace sbp {
namespace {

// x ghost width of the pools: R rounded up to an even count, so that every TMA
// box of a subdomain starts on a 16-byte boundary (the fixed-point tile's HX).
constexpr int ghost_x(int order) { return ((order / 2 + 1) / 2) * 2; }

struct DecompParams {
  int NX, NY, sw, col0, px, py;
  const FxSub* subs;
};

// Ghost update of the stage input: blockIdx.y = subdomain, blockIdx.z = side
// (0 west, 1 east, 2 south, 3 north); each thread copies scalars of the sw lines
// next to that side from the neighbour's interior.
__global__ void decomp_halo_kernel(const __grid_constant__ DecompParams P, double* pool) {
  const int b = blockIdx.y, side = blockIdx.z, sw = P.sw;
  const int bx = b % P.px, by = b / P.px;
  const int nbx = side == 0 ? bx - 1 : (side == 1 ? bx + 1 : bx);
  const int nby = side == 2 ? by - 1 : (side == 3 ? by + 1 : by);
  if (nbx < 0 || nbx >= P.px || nby < 0 || nby >= P.py) return;
  const FxSub S = P.subs[b], N = P.subs[nby * P.px + nbx];
  const int len = side < 2 ? S.ny : S.nx;
  const long long total = 3LL * sw * len;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(idx / ((long long)sw * len));
    const int rem = (int)(idx - (long long)c * sw * len);
    const int g = rem / len, p = rem - g * len;
    int di, dj, si, sj;  // destination (ghost) and source (neighbour interior) local indices
    if (side == 0) { di = -sw + g; dj = p; si = N.nx - sw + g; sj = p; }
    else if (side == 1) { di = S.nx + g; dj = p; si = g; sj = p; }
    else if (side == 2) { di = p; dj = -sw + g; si = p; sj = N.ny - sw + g; }
    else { di = p; dj = S.ny + g; si = p; sj = g; }
    pool[S.base + c * S.plane + (dj + sw) * S.pitch + (di + P.col0)] =
        pool[N.base + c * N.plane + (sj + sw) * N.pitch + (si + P.col0)];
  }
}

// Global AoS <-> subdomain SoA interiors: one thread per global point.
__global__ void decomp_scatter_kernel(const __grid_constant__ DecompParams P, const int* __restrict__ xsub,
                                      const int* __restrict__ ysub, const double* aos_in, double* aos_out,
                                      double* pool) {
  const long long n = (long long)P.NX * P.NY;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
    const int J = (int)(g / P.NX), I = (int)(g - (long long)J * P.NX);
    const int bx = xsub[I], by = ysub[J];
    const FxSub S = P.subs[by * P.px + bx];
    const long long q = S.base + (long long)(J - S.yoff + P.sw) * S.pitch + (I - S.xoff + P.col0);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      if (aos_in)
        pool[q + c * S.plane] = aos_in[3 * g + c];
      else
        aos_out[3 * g + c] = pool[q + c * S.plane];
    }
  }
}

// The stage kernels of a decomposed grid: the fixed-point FP64 stage kernel over
// the subdomains' tile list (wave_fixed_kernel<ORD, STAGE, true>).
template <int ORD, int STAGE>
cudaError_t launch_dec_one(const WaveParams<double>& prm, unsigned grid, cudaStream_t s) {
  using Tile = WaveStageTile<double, ORD, WK_HOM, STAGE>;
  static_assert(Tile::FIX && Tile::CONV > 0, "the decomposed path runs the converter-warp kernel");
  static_assert(Tile::HX == ghost_x(ORD), "pool x ghost width and tile halo must agree");
  CUtensorMap none;
  std::memset(&none, 0, sizeof(none));
  wave_fixed_kernel<ORD, STAGE, true><<<grid, fx_kernel_threads<Tile, true>(), Tile::SMEM, s>>>(
      none, none, none, none, none, none, none, prm);
  return cudaGetLastError();
}

template <int ORD>
cudaError_t launch_dec(int stage, const WaveParams<double>& prm, unsigned grid, cudaStream_t s) {
  switch (stage) {
    case ST_RHS: return launch_dec_one<ORD, ST_RHS>(prm, grid, s);
    case ST_FIRST: return launch_dec_one<ORD, ST_FIRST>(prm, grid, s);
    case ST_MID: return launch_dec_one<ORD, ST_MID>(prm, grid, s);
    case ST_LAST: return launch_dec_one<ORD, ST_LAST>(prm, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

template <int ORD, int STAGE>
cudaError_t configure_dec_one() {
  return cudaFuncSetAttribute(wave_fixed_kernel<ORD, STAGE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              WaveStageTile<double, ORD, WK_HOM, STAGE>::SMEM);
}

template <int ORD>
cudaError_t configure_dec() {
  cudaError_t e;
  if ((e = configure_dec_one<ORD, ST_RHS>()) != cudaSuccess) return e;
  if ((e = configure_dec_one<ORD, ST_FIRST>()) != cudaSuccess) return e;
  if ((e = configure_dec_one<ORD, ST_MID>()) != cudaSuccess) return e;
  return configure_dec_one<ORD, ST_LAST>();
}

template <int ORD> constexpr int dec_tile_rows() { return WaveStageTile<double, ORD, WK_HOM, ST_MID>::TY; }

}  // namespace
}  // namespace sbp

using namespace sbp;

struct sbp_decomp {
  sbp_desc d{};
  int px = 1, py = 1, sw = 1, col0 = 2, ty = 14;
  DecompParams prm{};
  WaveParams<double> wprm{};  // the stage-independent fields of the stage kernels' parameters
  std::vector<FxSub> subs;
  FxSub* d_subs = nullptr;
  FxTile* d_tiles = nullptr;
  unsigned char* d_tinfo = nullptr;  // per tile its geometry block (kFxTileInfoBytes each)
  CUtensorMap* d_maps = nullptr;  // [3 input buffers: un, wa, wb][sub][p, u, v], then [sub][u^n, acc]
  int ntiles = 0, maxlen = 0;
  int* d_xsub = nullptr;
  int* d_ysub = nullptr;
  int* d_err = nullptr;    // the stage kernels' error word
  int* d_sched = nullptr;  // their dynamic tile queue
  long long pool = 0;  // elements per state pool
  double *un = nullptr, *acc = nullptr, *wa = nullptr, *wb = nullptr, *io = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::map<long long, cudaGraphExec_t> graphs;  // per chunk length, the chunk's RK4 steps
  double graph_dt = 0.0;                         // the time step the graphs were captured with
  std::string msg;
};

namespace {

thread_local std::string g_decomp_create_error;  // the message of this thread's last failed sbp_decomp_create

int dfail(sbp_decomp* c, int code, const std::string& m) {
  if (c) c->msg = m;
  return code;
}

void release(sbp_decomp* c) {
  for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
  c->graphs.clear();
  cudaFree(c->d_subs);
  cudaFree(c->d_tiles);
  cudaFree(c->d_tinfo);
  cudaFree(c->d_maps);
  cudaFree(c->d_xsub);
  cudaFree(c->d_ysub);
  cudaFree(c->d_err);
  cudaFree(c->d_sched);
  cudaFree(c->un);
  cudaFree(c->acc);
  cudaFree(c->wa);
  cudaFree(c->wb);
  cudaFree(c->io);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
}

void decomp_taps(DirTaps<double>& t, int order, double scale) {
  const ops::Operator& op = ops::get(order);
  std::memset(&t, 0, sizeof(t));
  for (int s = 0; s < op.width; s++) t.taps[s] = scale * op.interior[s];
  for (int r = 0; r < op.cls_sz; r++)
    for (int s = 0; s < op.cls_width; s++) t.cls[r][s] = scale * op.closure[r][s];
}

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

// One 3-component tensor map over subdomain S's arrays (ghosts included) in buffer buf.
bool encode_sub(EncodeTiledFn enc, double* buf, const FxSub& S, int col0, int sw, const cuuint32_t box[3],
                CUtensorMap* out) {
  const cuuint64_t dims[3] = {(cuuint64_t)(S.nx + 2 * col0), (cuuint64_t)(S.ny + 2 * sw), 3};
  const cuuint64_t strides[2] = {(cuuint64_t)(S.pitch * 8), (cuuint64_t)(S.plane * 8)};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, buf + S.base, dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

cudaError_t halo(sbp_decomp* c, double* pool) {
  const int threads = 256;
  const long long total = 3LL * c->sw * c->maxlen;
  const unsigned bx = (unsigned)((total + threads - 1) / threads < 64 ? (total + threads - 1) / threads : 64);
  decomp_halo_kernel<<<dim3(bx, c->px * c->py, 4), threads, 0, c->stream>>>(c->prm, pool);
  return cudaGetLastError();
}

// One stage over every subdomain; in is one of un, wa, wb (its maps are chosen by it).
cudaError_t stage(sbp_decomp* c, int st, const double* in, double* wout, double* kout, double c_acc, double c_w) {
  WaveParams<double> p = c->wprm;
  p.in = in;
  p.wout = wout;
  p.kout = kout;
  p.c_acc = c_acc;
  p.c_w = c_w;
  set_fixed_scales(p, c->d.order, p.hix, p.hiy);
  const int nsub = c->px * c->py;
  const int which = in == c->un ? 0 : (in == c->wa ? 1 : 2);
  p.dmaps_in = c->d_maps + (long long)which * 3 * nsub;
  p.dmaps_na = c->d_maps + 9LL * nsub;
  const int nsm = device_sm_count();
  const unsigned grid = (unsigned)(c->ntiles < nsm ? c->ntiles : nsm);
  const int o = c->d.order;
  return o == 2 ? launch_dec<2>(st, p, grid, c->stream)
                : (o == 4 ? launch_dec<4>(st, p, grid, c->stream) : launch_dec<6>(st, p, grid, c->stream));
}

// AoS -> the subdomains' interiors (aos_in) or back (aos_out); one of them is null.
cudaError_t scatter(sbp_decomp* c, const double* aos_in, double* aos_out, double* pool) {
  const long long n = c->d.nx * c->d.ny;
  const unsigned blocks = (unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  decomp_scatter_kernel<<<blocks, 256, 0, c->stream>>>(c->prm, c->d_xsub, c->d_ysub, aos_in, aos_out, pool);
  return cudaGetLastError();
}

// One classical RK4 step (code/include/time_stepping/time_stepping.h:127-142). Each
// stage writes the ghost lines of the next stage's input as it produces the values
// (the fused exchange of wave_tile_fixed); u^n's ghosts must be current on entry.
cudaError_t enqueue_step(sbp_decomp* c, double dt) {
  cudaError_t e;
  if ((e = stage(c, ST_FIRST, c->un, c->wa, nullptr, dt / 6, 0.5 * dt)) != cudaSuccess) return e;
  if ((e = stage(c, ST_MID, c->wa, c->wb, nullptr, dt / 3, 0.5 * dt)) != cudaSuccess) return e;
  if ((e = stage(c, ST_MID, c->wb, c->wa, nullptr, dt / 3, dt)) != cudaSuccess) return e;
  return stage(c, ST_LAST, c->wa, nullptr, nullptr, dt / 6, 0.0);
}

#define DCK(call)                                                              \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) return dfail(c, SBP_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

// Synchronises the stream and reads (and clears) the stage kernels' error word.
int finish(sbp_decomp* c) {
  int h = 0;
  DCK(cudaMemcpyAsync(&h, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  DCK(cudaStreamSynchronize(c->stream));
  if (h) {
    DCK(cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
    DCK(cudaStreamSynchronize(c->stream));
    return dfail(c, SBP_ERR_DEVICE, "a bounded wait ran out in a stage kernel");
  }
  return SBP_OK;
}

}  // namespace

extern "C" {

int sbp_decomp_create(const sbp_desc* desc, int px, int py, sbp_decomp** out) {
  auto reject = [](int code, const char* why) {
    g_decomp_create_error = why;
    return code;
  };
  if (!desc || !out) return reject(SBP_ERR_INVALID, "null description or output");
  *out = nullptr;
  if (desc->problem != SBP_WAVE_HOM_2D) return reject(SBP_ERR_UNSUPPORTED, "only SBP_WAVE_HOM_2D is decomposed");
  if (desc->precision != SBP_FP64) return reject(SBP_ERR_UNSUPPORTED, "the decomposed path is FP64");
  if (desc->order != 2 && desc->order != 4 && desc->order != 6) return reject(SBP_ERR_INVALID, "order must be 2, 4 or 6");
  const ops::Operator& op = ops::get(desc->order);
  const long long NX = desc->nx, NY = desc->ny;
  if (px < 1 || py < 1 || px > 64 || py > 64) return reject(SBP_ERR_INVALID, "px, py must be in [1, 64]");
  // the whole grid at least the operator's minimum size, as sbp_create demands: below
  // it the left and right closure blocks would overlap
  const long long m = ops::min_points(desc->order);
  if (NX < m || NY < m) return reject(SBP_ERR_INVALID, "grid smaller than the operator's minimum size");
  // every subdomain at least one closure block wide (it then holds the closure
  // lines of a physical boundary and the ghost lines its neighbour needs)
  if (NX / px < op.cls_width || NY / py < op.cls_width || NX > (1 << 20) || NY > (1 << 20))
    return reject(SBP_ERR_INVALID, "subdomains narrower than the closure width, or grid above 2^20 per direction");
  if (!(desc->xr[0] > desc->xl[0]) || !(desc->xr[1] > desc->xl[1])) return reject(SBP_ERR_INVALID, "empty domain");
  EncodeTiledFn enc = encode_fn();
  if (!enc) return reject(SBP_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  sbp_decomp* c = new (std::nothrow) sbp_decomp;
  if (!c) return reject(SBP_ERR_CUDA, "host allocation");
  c->d = *desc;
  c->px = px;
  c->py = py;
  c->sw = (op.width - 1) / 2;
  c->col0 = ghost_x(desc->order);
  c->ty = desc->order == 2 ? dec_tile_rows<2>() : (desc->order == 4 ? dec_tile_rows<4>() : dec_tile_rows<6>());
  auto cfail = [&](int code, const char* why) {
    release(c);
    delete c;
    g_decomp_create_error = why;
    return code;
  };
  if (cudaSetDevice(desc->device) != cudaSuccess) return cfail(SBP_ERR_CUDA, "cudaSetDevice");
  if (desc->stream) {
    c->stream = (cudaStream_t)desc->stream;
  } else {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
      return cfail(SBP_ERR_CUDA, "cudaStreamCreate");
    c->own_stream = true;
  }
  // splits: subdomain b along x covers [b NX / px, (b + 1) NX / px). Each subdomain's
  // arrays: R ghost rows, col0 ghost columns (R rounded up to even), a row pitch of a
  // multiple of 32 doubles, planes starting at multiples of the pitch (TMA wants
  // 16-byte aligned bases, strides and x coordinates).
  std::vector<int> xsub(NX), ysub(NY);
  long long off = 0;
  for (int by = 0; by < py; by++)
    for (int bx = 0; bx < px; bx++) {
      FxSub s{};
      s.xoff = (int)(bx * NX / px);
      s.yoff = (int)(by * NY / py);
      s.nx = (int)((bx + 1) * NX / px) - s.xoff;
      s.ny = (int)((by + 1) * NY / py) - s.yoff;
      s.pitch = (s.nx + 2 * c->col0 + 31) / 32 * 32;
      s.plane = (long long)(s.ny + 2 * c->sw) * s.pitch;
      s.base = off;
      s.nbr[0] = bx > 0 ? by * px + bx - 1 : -1;
      s.nbr[1] = bx < px - 1 ? by * px + bx + 1 : -1;
      s.nbr[2] = by > 0 ? (by - 1) * px + bx : -1;
      s.nbr[3] = by < py - 1 ? (by + 1) * px + bx : -1;
      off += 3 * s.plane;
      c->subs.push_back(s);
      c->maxlen = std::max(c->maxlen, std::max(s.nx, s.ny));
    }
  c->pool = off;
  for (int bx = 0; bx < px; bx++)
    for (long long i = bx * NX / px; i < (bx + 1) * NX / px; i++) xsub[i] = bx;
  for (int by = 0; by < py; by++)
    for (long long j = by * NY / py; j < (by + 1) * NY / py; j++) ysub[j] = by;
  std::vector<FxTile> tiles;
  for (int b = 0; b < px * py; b++)
    for (int j0 = 0; j0 < c->subs[b].ny; j0 += c->ty)
      for (int i0 = 0; i0 < c->subs[b].nx; i0 += kWaveTX) tiles.push_back(FxTile{b, i0, j0, 0});
  c->ntiles = (int)tiles.size();
  const int nsub = px * py;
  // each tile's geometry block: the compute warps' FxGeom, the tile origin and the
  // neighbours' arrays the fused exchange writes into
  std::vector<unsigned char> tinfo(tiles.size() * kFxTileInfoBytes, 0);
  for (size_t t = 0; t < tiles.size(); t++) {
    const FxSub& S = c->subs[tiles[t].sub];
    FxTileInfo info{};
    info.g = FxGeom{S.nx, S.ny, S.xoff, S.yoff, c->col0, c->sw, S.pitch, S.plane, S.base};
    info.i0 = tiles[t].i0;
    info.j0 = tiles[t].j0;
    for (int side = 0; side < 4; side++) {
      info.nb[side] = FxNbr{0, 0, 0, -1, 0};
      if (S.nbr[side] >= 0) {
        const FxSub& N = c->subs[S.nbr[side]];
        info.nb[side] = FxNbr{N.base, N.pitch, N.plane, side < 2 ? N.nx : N.ny, 0};
      }
    }
    std::memcpy(&tinfo[t * kFxTileInfoBytes], &info, sizeof(info));
  }
  const size_t bytes = (size_t)c->pool * sizeof(double);
  if (cudaMalloc(&c->d_subs, c->subs.size() * sizeof(FxSub)) != cudaSuccess ||
      cudaMalloc(&c->d_tiles, tiles.size() * sizeof(FxTile)) != cudaSuccess ||
      cudaMalloc(&c->d_tinfo, tinfo.size()) != cudaSuccess ||
      cudaMalloc(&c->d_maps, 11 * (size_t)nsub * sizeof(CUtensorMap)) != cudaSuccess ||
      cudaMalloc(&c->d_xsub, NX * sizeof(int)) != cudaSuccess || cudaMalloc(&c->d_ysub, NY * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&c->d_err, sizeof(int)) != cudaSuccess || cudaMalloc(&c->d_sched, 2 * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&c->un, bytes) != cudaSuccess || cudaMalloc(&c->acc, bytes) != cudaSuccess ||
      cudaMalloc(&c->wa, bytes) != cudaSuccess || cudaMalloc(&c->wb, bytes) != cudaSuccess ||
      cudaMalloc(&c->io, (size_t)NX * NY * 3 * sizeof(double)) != cudaSuccess)
    return cfail(SBP_ERR_CUDA, "cudaMalloc");
  // TMA maps per subdomain: the p/u/v boxes of each possible stage input, then u^n and acc
  const int HX = c->col0, HY = c->sw, TY = c->ty;
  const cuuint32_t boxP[3] = {(cuuint32_t)(kWaveTX + 2 * HX), (cuuint32_t)(TY + 2 * HY), 1};
  const cuuint32_t boxU[3] = {(cuuint32_t)(kWaveTX + 2 * HX), (cuuint32_t)TY, 1};
  const cuuint32_t boxV[3] = {(cuuint32_t)kWaveTX, (cuuint32_t)(TY + 2 * HY), 1};
  const cuuint32_t boxPt[3] = {(cuuint32_t)kWaveTX, (cuuint32_t)TY, 3};
  std::vector<CUtensorMap> maps(11 * (size_t)nsub);
  double* inbufs[3] = {c->un, c->wa, c->wb};
  bool ok = true;
  for (int w = 0; w < 3; w++)
    for (int b = 0; b < nsub; b++) {
      CUtensorMap* mm = &maps[((size_t)w * nsub + b) * 3];
      ok = ok && encode_sub(enc, inbufs[w], c->subs[b], c->col0, c->sw, boxP, &mm[0]) &&
           encode_sub(enc, inbufs[w], c->subs[b], c->col0, c->sw, boxU, &mm[1]) &&
           encode_sub(enc, inbufs[w], c->subs[b], c->col0, c->sw, boxV, &mm[2]);
    }
  for (int b = 0; b < nsub; b++) {
    CUtensorMap* mm = &maps[9 * (size_t)nsub + 2 * (size_t)b];
    ok = ok && encode_sub(enc, c->un, c->subs[b], c->col0, c->sw, boxPt, &mm[0]) &&
         encode_sub(enc, c->acc, c->subs[b], c->col0, c->sw, boxPt, &mm[1]);
  }
  if (!ok) return cfail(SBP_ERR_CUDA, "cuTensorMapEncodeTiled failed for a subdomain");
  // zeroed pools: ghost cells outside the grid are never used, but stay defined
  if (cudaMemset(c->un, 0, bytes) != cudaSuccess || cudaMemset(c->acc, 0, bytes) != cudaSuccess ||
      cudaMemset(c->wa, 0, bytes) != cudaSuccess || cudaMemset(c->wb, 0, bytes) != cudaSuccess ||
      cudaMemset(c->d_err, 0, sizeof(int)) != cudaSuccess || cudaMemset(c->d_sched, 0, 2 * sizeof(int)) != cudaSuccess ||
      cudaMemcpy(c->d_subs, c->subs.data(), c->subs.size() * sizeof(FxSub), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(c->d_tiles, tiles.data(), tiles.size() * sizeof(FxTile), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(c->d_tinfo, tinfo.data(), tinfo.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(c->d_maps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(c->d_xsub, xsub.data(), NX * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(c->d_ysub, ysub.data(), NY * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
    return cfail(SBP_ERR_CUDA, "set-up copies");
  const cudaError_t ce =
      desc->order == 2 ? configure_dec<2>() : (desc->order == 4 ? configure_dec<4>() : configure_dec<6>());
  if (ce != cudaSuccess) return cfail(SBP_ERR_CUDA, "shared-memory opt-in of the stage kernels");
  if (cudaDeviceSynchronize() != cudaSuccess) return cfail(SBP_ERR_CUDA, "set-up");
  const double hix = (NX - 1) / (desc->xr[0] - desc->xl[0]), hiy = (NY - 1) / (desc->xr[1] - desc->xl[1]);
  DecompParams& P = c->prm;
  P.NX = (int)NX;
  P.NY = (int)NY;
  P.sw = c->sw;
  P.col0 = c->col0;
  P.px = px;
  P.py = py;
  P.subs = c->d_subs;
  WaveParams<double>& W = c->wprm;
  std::memset(&W, 0, sizeof(W));
  W.nx = (int)NX;  // the global grid: closure regions and SAT faces
  W.ny = (int)NY;
  W.un = c->un;
  W.acc = c->acc;
  decomp_taps(W.dx, desc->order, -hix);
  decomp_taps(W.dy, desc->order, -hiy);
  W.bwx = hix * op.hinv0;
  W.bwy = hiy * op.hinv0;
  W.bc = desc->bc == SBP_BC_CHARACTERISTIC ? BC_CHARACTERISTIC : BC_FREE_SURFACE;
  W.hix = hix;
  W.hiy = hiy;
  W.err = c->d_err;
  W.sched = c->d_sched;
  W.dtiles = c->d_tiles;
  W.dtinfo = c->d_tinfo;
  W.dsubs = c->d_subs;
  W.dntiles = c->ntiles;
  *out = c;
  return SBP_OK;
}

int sbp_decomp_destroy(sbp_decomp* c) {
  if (!c) return SBP_ERR_INVALID;
  cudaSetDevice(c->d.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  release(c);
  delete c;
  return SBP_OK;
}

const char* sbp_decomp_last_error(const sbp_decomp* c) { return c ? c->msg.c_str() : g_decomp_create_error.c_str(); }

int sbp_decomp_set_state(sbp_decomp* c, const double* aos, int where) {
  if (!c || !aos) return SBP_ERR_INVALID;
  if (where != SBP_HOST && where != SBP_DEVICE)
    return dfail(c, SBP_ERR_INVALID, "where must be SBP_HOST or SBP_DEVICE");
  cudaSetDevice(c->d.device);
  const size_t bytes = (size_t)c->d.nx * c->d.ny * 3 * sizeof(double);
  const double* src = aos;
  if (where == SBP_HOST) {
    DCK(cudaMemcpyAsync(c->io, aos, bytes, cudaMemcpyHostToDevice, c->stream));
    src = c->io;
  }
  DCK(scatter(c, src, nullptr, c->un));
  DCK(cudaStreamSynchronize(c->stream));
  return SBP_OK;
}

int sbp_decomp_get_state(sbp_decomp* c, double* aos, int where) {
  if (!c || !aos) return SBP_ERR_INVALID;
  if (where != SBP_HOST && where != SBP_DEVICE)
    return dfail(c, SBP_ERR_INVALID, "where must be SBP_HOST or SBP_DEVICE");
  cudaSetDevice(c->d.device);
  const size_t bytes = (size_t)c->d.nx * c->d.ny * 3 * sizeof(double);
  double* dst = where == SBP_HOST ? c->io : aos;
  DCK(scatter(c, nullptr, dst, c->un));
  if (where == SBP_HOST) DCK(cudaMemcpyAsync(aos, c->io, bytes, cudaMemcpyDeviceToHost, c->stream));
  DCK(cudaStreamSynchronize(c->stream));
  return SBP_OK;
}

int sbp_decomp_rhs(sbp_decomp* c, const double* src, double* dst, int where) {
  if (!c || !src || !dst) return SBP_ERR_INVALID;
  if (where != SBP_HOST && where != SBP_DEVICE)
    return dfail(c, SBP_ERR_INVALID, "where must be SBP_HOST or SBP_DEVICE");
  cudaSetDevice(c->d.device);
  const size_t bytes = (size_t)c->d.nx * c->d.ny * 3 * sizeof(double);
  if (where == SBP_HOST) {
    DCK(cudaMemcpyAsync(c->io, src, bytes, cudaMemcpyHostToDevice, c->stream));
    DCK(scatter(c, c->io, nullptr, c->wa));
  } else {
    DCK(scatter(c, src, nullptr, c->wa));
  }
  DCK(halo(c, c->wa));
  DCK(stage(c, ST_RHS, c->wa, nullptr, c->wb, 0.0, 0.0));
  if (where == SBP_HOST) {
    DCK(scatter(c, nullptr, c->io, c->wb));
    DCK(cudaMemcpyAsync(dst, c->io, bytes, cudaMemcpyDeviceToHost, c->stream));
  } else {
    DCK(scatter(c, nullptr, dst, c->wb));
  }
  return finish(c);
}

int sbp_decomp_rk4_resident(sbp_decomp* c, double dt, long long nsteps) {
  if (!c || nsteps < 0 || !(dt > 0)) return SBP_ERR_INVALID;
  cudaSetDevice(c->d.device);
  // u^n's ghost lines from its neighbours once (after sbp_decomp_set_state they are
  // stale); from there each stage keeps the next stage input's ghosts current
  DCK(halo(c, c->un));
  // chunks of up to 50 steps, each length captured once as a CUDA graph (4 launches a
  // step); a new time step drops the graphs
  const long long chunk = 50;
  if (c->graph_dt != dt) {
    for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
    c->graphs.clear();
    c->graph_dt = dt;
  }
  long long left = nsteps;
  while (left > 0) {
    const long long n = left < chunk ? left : chunk;
    auto it = c->graphs.find(n);
    if (it == c->graphs.end()) {
      cudaGraph_t g = nullptr;
      DCK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t e = cudaSuccess;
      for (long long k = 0; k < n && e == cudaSuccess; k++) e = enqueue_step(c, dt);
      const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
      if (e != cudaSuccess || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return dfail(c, SBP_ERR_CUDA, cudaGetErrorString(e != cudaSuccess ? e : ce));
      }
      cudaGraphExec_t ex = nullptr;
      const cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
      cudaGraphDestroy(g);
      DCK(ie);
      it = c->graphs.emplace(n, ex).first;
    }
    DCK(cudaGraphLaunch(it->second, c->stream));
    left -= n;
  }
  return finish(c);
}

}  // extern "C"
