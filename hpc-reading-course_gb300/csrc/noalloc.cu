// noalloc.cu -- sbp_wave_rhs_noalloc: the 2D acoustic-wave RHS evaluation of
// sbp_rhs without any device allocation.
//
// sbp_rhs works on a context whose structure-of-arrays staging buffers come
// from cudaMalloc. Some callers cannot allocate: a host framework that owns
// all device memory through its own pool and forbids plugins to call
// cudaMalloc, or a caller inside a latency-bound loop that cannot take
// cudaMalloc's implicit device synchronisation. For them this entry point
// keeps its scratch -- the input and output component planes and an error
// word -- in one file-scope static device array of fixed size, which every
// GPU that loads the library holds until the process exits. The caller passes
// its own device input and output arrays.
//
// Limits and sharing rules:
//   * grids with roundup(nx, 64) * ny <= SBP_NOALLOC_MAX_PLANE points;
//     larger grids are rejected with SBP_ERR_TOO_LARGE before any GPU work;
//   * every call on a device uses the same array and leaves its contents
//     behind; the error word is cleared at the start of each call; two calls
//     whose GPU work overlaps (different streams or threads) race on the
//     array and give wrong results -- serialise them;
//   * the first call on a device does a one-time set-up on that device (the
//     array's device address and the stage kernels' shared-memory opt-in);
//     make that first call before any stream capture. Later calls look the
//     address up again (no allocation) and redo the set-up if it moved, as it
//     can after cudaDeviceReset reloads the module;
//   * every call is synchronous: it waits on its stream for its own work and
//     reads the kernel's error word back before it returns;
//   * the calling thread's current device is the same on return as on entry.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/sbpgpu.h"
#include "launch.h"
#include "sbp_ops.h"

using namespace sbp;

namespace {

constexpr long long kPlane = SBP_NOALLOC_MAX_PLANE;
// Input planes (3), output planes (3), then 32 doubles holding the error word.
constexpr long long kScratchDoubles = 6 * kPlane + 32;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {nullptr};

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Set-up per device, with that device current: the device address of the
// static array (host code may not use the symbol itself as a pointer) and the
// shared-memory opt-in of the FP64 stage kernels. The opt-in runs once per
// device; the address is looked up on every call (cheap, allocates nothing)
// so that a module reloaded after cudaDeviceReset never gets a stale address,
// and a changed address repeats the opt-in on the reloaded module.
int setup_device(int device, double** scratch) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  double* ptr = nullptr;
  if (cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return SBP_ERR_CUDA;
  if (g_scratch_addr[device] != ptr) {
    for (int order : {2, 4, 6})
      if (configure_wave<double>(order, WK_HOM) != cudaSuccess) return SBP_ERR_CUDA;
    g_scratch_addr[device] = ptr;
  }
  *scratch = ptr;
  return SBP_OK;
}

// Puts the caller's current device back on every return path.
struct DeviceRestore {
  int dev = -1;
  DeviceRestore() {
    if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
  }
  ~DeviceRestore() {
    if (dev >= 0) cudaSetDevice(dev);
  }
};

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

void fill(DirTaps<double>& t, int order, double scale) {
  const ops::Operator& op = ops::get(order);
  std::memset(&t, 0, sizeof(t));
  for (int s = 0; s < op.width; s++) t.taps[s] = scale * op.interior[s];
  for (int r = 0; r < op.cls_sz; r++)
    for (int s = 0; s < op.cls_width; s++) t.cls[r][s] = scale * op.closure[r][s];
}

// Status codes carry the reason: this entry point has no context to hold a message.
int reject(int code, const char*) { return code; }

}  // namespace

extern "C" int sbp_wave_rhs_noalloc(const sbp_desc* d, double t, const double* src, double* dst) {
  if (!d || !src || !dst) return reject(SBP_ERR_INVALID, "null argument");
  if (d->problem != SBP_WAVE_HOM_2D) return reject(SBP_ERR_INVALID, "only SBP_WAVE_HOM_2D is provided");
  if (d->precision != SBP_FP64) return reject(SBP_ERR_INVALID, "only SBP_FP64 is provided");
  if (d->order != 2 && d->order != 4 && d->order != 6) return reject(SBP_ERR_INVALID, "order must be 2, 4 or 6");
  if (d->bc != SBP_BC_REFERENCE && d->bc != SBP_BC_CHARACTERISTIC)
    return reject(SBP_ERR_INVALID, "unknown boundary treatment");
  const long long m = ops::min_points(d->order);
  if (d->nx < m || d->ny < m) return reject(SBP_ERR_INVALID, "grid smaller than the operator's minimum size");
  if (!(d->xr[0] > d->xl[0]) || !(d->xr[1] > d->xl[1])) return reject(SBP_ERR_INVALID, "empty domain");
  const long long nx = d->nx, ny = d->ny;
  const long long pitch = (nx + 63) / 64 * 64;
  if (pitch > kPlane || pitch * ny > kPlane)
    return reject(SBP_ERR_TOO_LARGE,
                  "grid exceeds the static scratch: roundup(nx, 64) * ny must be <= SBP_NOALLOC_MAX_PLANE");
  if (d->device < 0 || d->device >= kMaxDevices) return reject(SBP_ERR_INVALID, "device ordinal out of range");
  const DeviceRestore restore;
  if (cudaSetDevice(d->device) != cudaSuccess) return reject(SBP_ERR_CUDA, "cudaSetDevice failed");
  double* scratch = nullptr;
  if (setup_device(d->device, &scratch)) return reject(SBP_ERR_CUDA, "set-up of the static scratch failed");
  EncodeTiledFn enc = encode_fn();
  if (!enc) return reject(SBP_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");

  const long long plane = pitch * ny;
  double* in = scratch;
  double* out = scratch + 3 * kPlane;
  int* err = reinterpret_cast<int*>(scratch + 6 * kPlane);
  cudaStream_t s = (cudaStream_t)d->stream;

  // TMA descriptors of the input planes (host-side encode, no allocation)
  const int R = d->order / 2, HX = (R + 1) / 2 * 2, HY = R;
  const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, 3};
  const cuuint64_t strides[2] = {(cuuint64_t)(pitch * 8), (cuuint64_t)(plane * 8)};
  const cuuint32_t estr[3] = {1, 1, 1};
  const int TY = wave_tile_height(8);
  const cuuint32_t boxP[3] = {(cuuint32_t)(kWaveTX + 2 * HX), (cuuint32_t)(TY + 2 * HY), 1};
  const cuuint32_t boxU[3] = {(cuuint32_t)(kWaveTX + 2 * HX), (cuuint32_t)TY, 1};
  const cuuint32_t boxV[3] = {(cuuint32_t)kWaveTX, (cuuint32_t)(TY + 2 * HY), 1};
  WaveMaps maps;
  CUtensorMap* mp[3] = {&maps.p, &maps.u, &maps.v};
  const cuuint32_t* boxes[3] = {boxP, boxU, boxV};
  for (int k = 0; k < 3; k++)
    if (enc(mp[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, in, dims, strides, boxes[k], estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return reject(SBP_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  maps.n = maps.a = maps.c = maps.k = maps.p;  // the RHS-only stage loads no per-point operands

  WaveParams<double> p;
  std::memset(&p, 0, sizeof(p));
  p.nx = (int)nx;
  p.ny = (int)ny;
  p.pitch = pitch;
  p.plane = plane;
  const double hix = (nx - 1) / (d->xr[0] - d->xl[0]), hiy = (ny - 1) / (d->xr[1] - d->xl[1]);
  fill(p.dx, d->order, -hix);
  fill(p.dy, d->order, -hiy);
  const double hi0 = ops::get(d->order).hinv0;
  p.bwx = hix * hi0;
  p.bwy = hiy * hi0;
  p.bc = d->bc == SBP_BC_CHARACTERISTIC ? BC_CHARACTERISTIC : BC_FREE_SURFACE;
  p.in = in;
  p.kout = out;
  p.t = t;
  p.err = err;
  set_fixed_scales(p, d->order, hix, hiy);

  // The error word must start at zero; everything else is overwritten.
  if (cudaMemsetAsync(err, 0, sizeof(int), s) != cudaSuccess) return reject(SBP_ERR_CUDA, "cudaMemsetAsync failed");
  if (launch_pack<double>(src, in, (int)nx, (int)ny, 3, pitch, plane, s) != cudaSuccess ||
      launch_wave<double>(d->order, WK_HOM, ST_RHS, maps, p, s) != cudaSuccess ||
      launch_unpack<double>(out, dst, (int)nx, (int)ny, 3, pitch, plane, s) != cudaSuccess)
    return reject(SBP_ERR_CUDA, "kernel launch failed");
  int h_err = 0;
  if (cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return reject(SBP_ERR_CUDA, "CUDA error while evaluating the RHS");
  if (h_err) return reject(SBP_ERR_DEVICE, "a TMA tile wait timed out in the stage kernel");
  return SBP_OK;
}
