// decomp.cu -- the 2D wave system (rho = K = 1, FP64) on a P x Q decomposition of
// one grid, on one GPU: each subdomain holds its own SoA state with sw = R ghost
// lines on each side, and every RK4 stage first copies the neighbours' edge lines
// into the ghosts (a halo-exchange kernel), then evaluates the RHS and the stage
// update of all subdomains in one launch. It is the reference's non-overlapped
// decomposed path -- rhs_local / rhs_all over a DMDA block grid
// (code/include/partitioned_rhs/rhs.h:97-181, 183-360) with the VecScatter ghost
// update of code/src/scatter/scatter_ctx.cpp:149-211 -- with the halo exchange
// on the device, the step towards one subdomain per GPU.
//
// Interior points of a subdomain evaluate the central stencil across internal
// edges from the ghosts; closure rows and SAT terms apply only at the physical
// boundary, so a subdomain at least one closure block wide holds every closure
// line it needs. The arithmetic per point is that of the single-grid path
// (d1_line / closure_line tap order, the wave_hom SAT in FP64), so a decomposed
// run matches the single grid to rounding.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/sbpgpu.h"
#include "launch.h"
#include "sbp_ops.h"

namespace sbp {
namespace {

struct DecompSub {
  int nx, ny;        // interior points
  int xoff, yoff;    // global index of the interior's first column / row
  long long pitch;   // elements per row, ghosts included
  long long plane;   // elements per component plane (ny + 2 sw rows)
  long long base;    // element offset of the subdomain's planes in a pool
};

struct DecompTile {
  int sub, i0, j0, pad;
};

struct DecompParams {
  int NX, NY, sw, bc, px, py;
  DirTaps<double> dx, dy;  // -hi * stencils
  double bwx, bwy;         // hi * HI[0]: SAT weights
  const DecompSub* subs;
};

constexpr int kDTX = 32, kDTY = 32, kDRows = 8;  // a CTA: 32 x 8 threads over a 32 x 32 tile

// D1 of a line held by one subdomain: the element of global index g is at
// base[(g - off) * st] (ghost cells included). Interior points use the central
// stencil; the closure rows (d1_line / closure_line order) need the line's first
// or last closure block inside the subdomain, which the width check guarantees.
template <int ORD>
__device__ __forceinline__ double d1_sub(const DirTaps<double>& d, const double* base, long long st, int off, int n,
                                         int I) {
  constexpr int W = OpShape<ORD>::W, CS = OpShape<ORD>::CS, CW = OpShape<ORD>::CW, R = (W - 1) / 2;
  if (I >= CS && I < n - CS) {
    const double* c = base + (long long)(I - R - off) * st;
    double s = d.taps[0] * c[0];
#pragma unroll
    for (int k = 1; k < W; k++)
      if (k != R) s = fma(d.taps[k], c[k * st], s);
    return s;
  }
  if (I < CS) {
    const double* c = base - (long long)off * st;  // off == 0: the first subdomain
    double s = d.cls[I][0] * c[0];
#pragma unroll
    for (int k = 1; k < CW; k++) s = fma(d.cls[I][k], c[k * st], s);
    return s;
  }
  const int r = n - 1 - I;
  const double* c = base + (long long)(n - CW - off) * st;
  double s = -d.cls[r][CW - 1] * c[0];
#pragma unroll
  for (int k = 1; k < CW; k++) s = fma(-d.cls[r][CW - 1 - k], c[k * st], s);
  return s;
}

// Ghost update of the stage input: blockIdx.y = subdomain, blockIdx.z = side
// (0 west, 1 east, 2 south, 3 north); each thread copies scalars of the sw lines
// next to that side from the neighbour's interior.
__global__ void decomp_halo_kernel(const __grid_constant__ DecompParams P, double* pool) {
  const int b = blockIdx.y, side = blockIdx.z, sw = P.sw;
  const int bx = b % P.px, by = b / P.px;
  const int nbx = side == 0 ? bx - 1 : (side == 1 ? bx + 1 : bx);
  const int nby = side == 2 ? by - 1 : (side == 3 ? by + 1 : by);
  if (nbx < 0 || nbx >= P.px || nby < 0 || nby >= P.py) return;
  const DecompSub S = P.subs[b], N = P.subs[nby * P.px + nbx];
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
    pool[S.base + c * S.plane + (dj + sw) * S.pitch + (di + sw)] =
        pool[N.base + c * N.plane + (sj + sw) * N.pitch + (si + sw)];
  }
}

template <int ORD, int STAGE>
__global__ void __launch_bounds__(kDTX * kDRows)
    decomp_stage_kernel(const __grid_constant__ DecompParams P, const DecompTile* __restrict__ tiles,
                        const double* __restrict__ in, double* un, double* acc, double* wout, double* kout,
                        const double c_acc, const double c_w) {
  const DecompTile t = tiles[blockIdx.x];
  const DecompSub S = P.subs[t.sub];
  const int sw = P.sw;
  const int i = t.i0 + threadIdx.x;
  if (i >= S.nx) return;
  const int I = S.xoff + i;
  const double* U = in + S.base;
  const double* V = U + S.plane;
  const double* Pp = V + S.plane;
#pragma unroll 1
  for (int r = 0; r < kDTY / kDRows; r++) {
    const int j = t.j0 + threadIdx.y + kDRows * r;
    if (j >= S.ny) continue;
    const int J = S.yoff + j;
    const long long row = (long long)(j + sw) * S.pitch + sw;  // local i = 0 of row j
    const long long col = (long long)sw * S.pitch + (i + sw);  // local j = 0 of column i
    const long long q = row + i;
    double ku = d1_sub<ORD>(P.dx, Pp + row, 1, S.xoff, P.NX, I);
    double kv = d1_sub<ORD>(P.dy, Pp + col, S.pitch, S.yoff, P.NY, J);
    double kp = d1_sub<ORD>(P.dx, U + row, 1, S.xoff, P.NX, I) + d1_sub<ORD>(P.dy, V + col, S.pitch, S.yoff, P.NY, J);
    const double uc = U[q], vc = V[q], pc = Pp[q];
    // SAT at the physical boundary (the wave_hom terms of the single-grid path, rho = K = 1)
    if (P.bc != BC_NONE && (I == 0 || J == 0 || I == P.NX - 1 || J == P.NY - 1)) {
      if (P.bc == BC_FREE_SURFACE) {
        if (I == 0) ku = ku - P.bwx * pc;
        if (J == 0) kv = kv - P.bwy * pc;
        if (I == P.NX - 1) ku = ku + P.bwx * pc;
        if (J == P.NY - 1) kv = kv + P.bwy * pc;
      } else {
        if (I == 0) { const double g = P.bwx * (pc + 1.0 * uc); ku -= 0.5 * g; kp -= 0.5 * g; }
        if (J == 0) { const double g = P.bwy * (pc + 1.0 * vc); kv -= 0.5 * g; kp -= 0.5 * g; }
        if (I == P.NX - 1) { const double g = P.bwx * (pc - 1.0 * uc); ku += 0.5 * g; kp -= 0.5 * g; }
        if (J == P.NY - 1) { const double g = P.bwy * (pc - 1.0 * vc); kv += 0.5 * g; kp -= 0.5 * g; }
      }
    }
    const double kc[3] = {ku, kv, kp}, cen[3] = {uc, vc, pc};
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const long long o = S.base + c * S.plane + q;
      if constexpr (STAGE == ST_RHS) {
        kout[o] = kc[c];
      } else if constexpr (STAGE == ST_FIRST) {
        acc[o] = fma(c_acc, kc[c], cen[c]);
        wout[o] = fma(c_w, kc[c], cen[c]);
      } else if constexpr (STAGE == ST_MID) {
        acc[o] = fma(c_acc, kc[c], acc[o]);
        wout[o] = fma(c_w, kc[c], un[o]);
      } else {
        un[o] = fma(c_acc, kc[c], acc[o]);
      }
    }
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
    const DecompSub S = P.subs[by * P.px + bx];
    const long long q = S.base + (long long)(J - S.yoff + P.sw) * S.pitch + (I - S.xoff + P.sw);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      if (aos_in)
        pool[q + c * S.plane] = aos_in[3 * g + c];
      else
        aos_out[3 * g + c] = pool[q + c * S.plane];
    }
  }
}

template <int ORD>
cudaError_t launch_stage_o(int stage, const DecompParams& P, const DecompTile* tiles, int ntiles, const double* in,
                           double* un, double* acc, double* wout, double* kout, double c_acc, double c_w,
                           cudaStream_t s) {
  const dim3 block(kDTX, kDRows);
  switch (stage) {
    case ST_RHS:
      decomp_stage_kernel<ORD, ST_RHS><<<ntiles, block, 0, s>>>(P, tiles, in, un, acc, wout, kout, c_acc, c_w);
      break;
    case ST_FIRST:
      decomp_stage_kernel<ORD, ST_FIRST><<<ntiles, block, 0, s>>>(P, tiles, in, un, acc, wout, kout, c_acc, c_w);
      break;
    case ST_MID:
      decomp_stage_kernel<ORD, ST_MID><<<ntiles, block, 0, s>>>(P, tiles, in, un, acc, wout, kout, c_acc, c_w);
      break;
    case ST_LAST:
      decomp_stage_kernel<ORD, ST_LAST><<<ntiles, block, 0, s>>>(P, tiles, in, un, acc, wout, kout, c_acc, c_w);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace
}  // namespace sbp

using namespace sbp;

struct sbp_decomp {
  sbp_desc d{};
  int px = 1, py = 1, sw = 1;
  DecompParams prm{};
  std::vector<DecompSub> subs;
  DecompSub* d_subs = nullptr;
  DecompTile* d_tiles = nullptr;
  int ntiles = 0, maxlen = 0;
  int* d_xsub = nullptr;
  int* d_ysub = nullptr;
  long long pool = 0;  // elements per state pool
  double *un = nullptr, *acc = nullptr, *wa = nullptr, *wb = nullptr, *io = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string msg;
};

namespace {

std::string g_decomp_create_error;  // the message of the last failed sbp_decomp_create

int dfail(sbp_decomp* c, int code, const std::string& m) {
  if (c) c->msg = m;
  return code;
}

void release(sbp_decomp* c) {
  cudaFree(c->d_subs);
  cudaFree(c->d_tiles);
  cudaFree(c->d_xsub);
  cudaFree(c->d_ysub);
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

cudaError_t halo(sbp_decomp* c, double* pool) {
  const int threads = 256;
  const long long total = 3LL * c->sw * c->maxlen;
  const unsigned bx = (unsigned)((total + threads - 1) / threads < 64 ? (total + threads - 1) / threads : 64);
  decomp_halo_kernel<<<dim3(bx, c->px * c->py, 4), threads, 0, c->stream>>>(c->prm, pool);
  return cudaGetLastError();
}

cudaError_t stage(sbp_decomp* c, int st, const double* in, double* wout, double* kout, double c_acc, double c_w) {
  const int o = c->d.order;
  const auto f = o == 2 ? launch_stage_o<2> : (o == 4 ? launch_stage_o<4> : launch_stage_o<6>);
  return f(st, c->prm, c->d_tiles, c->ntiles, in, c->un, c->acc, wout, kout, c_acc, c_w, c->stream);
}

// AoS -> the subdomains' interiors (aos_in) or back (aos_out); one of them is null.
cudaError_t scatter(sbp_decomp* c, const double* aos_in, double* aos_out, double* pool) {
  const long long n = c->d.nx * c->d.ny;
  const unsigned blocks = (unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  decomp_scatter_kernel<<<blocks, 256, 0, c->stream>>>(c->prm, c->d_xsub, c->d_ysub, aos_in, aos_out, pool);
  return cudaGetLastError();
}

#define DCK(call)                                                              \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) return dfail(c, SBP_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

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
  // every subdomain at least one closure block wide (it then holds the closure
  // lines of a physical boundary and the ghost lines its neighbour needs)
  // the whole grid at least the operator's minimum size, as sbp_create demands: below
  // it the left and right closure blocks would overlap
  const long long m = ops::min_points(desc->order);
  if (NX < m || NY < m) return reject(SBP_ERR_INVALID, "grid smaller than the operator's minimum size");
  if (NX / px < op.cls_width || NY / py < op.cls_width || NX > (1 << 20) || NY > (1 << 20))
    return reject(SBP_ERR_INVALID, "subdomains narrower than the closure width, or grid above 2^20 per direction");
  if (!(desc->xr[0] > desc->xl[0]) || !(desc->xr[1] > desc->xl[1])) return reject(SBP_ERR_INVALID, "empty domain");
  sbp_decomp* c = new (std::nothrow) sbp_decomp;
  if (!c) return reject(SBP_ERR_CUDA, "host allocation");
  c->d = *desc;
  c->px = px;
  c->py = py;
  c->sw = (op.width - 1) / 2;
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
  // splits: subdomain b along x covers [b NX / px, (b + 1) NX / px)
  std::vector<int> xsub(NX), ysub(NY);
  long long off = 0;
  for (int by = 0; by < py; by++)
    for (int bx = 0; bx < px; bx++) {
      DecompSub s{};
      s.xoff = (int)(bx * NX / px);
      s.yoff = (int)(by * NY / py);
      s.nx = (int)((bx + 1) * NX / px) - s.xoff;
      s.ny = (int)((by + 1) * NY / py) - s.yoff;
      s.pitch = (s.nx + 2 * c->sw + 31) / 32 * 32;
      s.plane = (long long)(s.ny + 2 * c->sw) * s.pitch;
      s.base = off;
      off += 3 * s.plane;
      c->subs.push_back(s);
      c->maxlen = std::max(c->maxlen, std::max(s.nx, s.ny));
    }
  c->pool = off;
  for (int bx = 0; bx < px; bx++)
    for (long long i = bx * NX / px; i < (bx + 1) * NX / px; i++) xsub[i] = bx;
  for (int by = 0; by < py; by++)
    for (long long j = by * NY / py; j < (by + 1) * NY / py; j++) ysub[j] = by;
  std::vector<DecompTile> tiles;
  for (int b = 0; b < px * py; b++)
    for (int j0 = 0; j0 < c->subs[b].ny; j0 += kDTY)
      for (int i0 = 0; i0 < c->subs[b].nx; i0 += kDTX) tiles.push_back(DecompTile{b, i0, j0, 0});
  c->ntiles = (int)tiles.size();
  const size_t bytes = (size_t)c->pool * sizeof(double);
  if (cudaMalloc(&c->d_subs, c->subs.size() * sizeof(DecompSub)) != cudaSuccess ||
      cudaMalloc(&c->d_tiles, tiles.size() * sizeof(DecompTile)) != cudaSuccess ||
      cudaMalloc(&c->d_xsub, NX * sizeof(int)) != cudaSuccess || cudaMalloc(&c->d_ysub, NY * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&c->un, bytes) != cudaSuccess || cudaMalloc(&c->acc, bytes) != cudaSuccess ||
      cudaMalloc(&c->wa, bytes) != cudaSuccess || cudaMalloc(&c->wb, bytes) != cudaSuccess ||
      cudaMalloc(&c->io, (size_t)NX * NY * 3 * sizeof(double)) != cudaSuccess)
    return cfail(SBP_ERR_CUDA, "cudaMalloc");
  // zeroed pools: ghost cells outside the grid are never read, but stay defined
  if (cudaMemset(c->un, 0, bytes) != cudaSuccess || cudaMemset(c->acc, 0, bytes) != cudaSuccess ||
      cudaMemset(c->wa, 0, bytes) != cudaSuccess || cudaMemset(c->wb, 0, bytes) != cudaSuccess ||
      cudaMemcpy(c->d_subs, c->subs.data(), c->subs.size() * sizeof(DecompSub), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(c->d_tiles, tiles.data(), tiles.size() * sizeof(DecompTile), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(c->d_xsub, xsub.data(), NX * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(c->d_ysub, ysub.data(), NY * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
    return cfail(SBP_ERR_CUDA, "set-up copies");
  const double hix = (NX - 1) / (desc->xr[0] - desc->xl[0]), hiy = (NY - 1) / (desc->xr[1] - desc->xl[1]);
  DecompParams& P = c->prm;
  P.NX = (int)NX;
  P.NY = (int)NY;
  P.sw = c->sw;
  P.px = px;
  P.py = py;
  P.bc = desc->bc == SBP_BC_CHARACTERISTIC ? BC_CHARACTERISTIC : BC_FREE_SURFACE;
  decomp_taps(P.dx, desc->order, -hix);
  decomp_taps(P.dy, desc->order, -hiy);
  P.bwx = hix * op.hinv0;
  P.bwy = hiy * op.hinv0;
  P.subs = c->d_subs;
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
  DCK(cudaStreamSynchronize(c->stream));
  return SBP_OK;
}

int sbp_decomp_rk4_resident(sbp_decomp* c, double dt, long long nsteps) {
  if (!c || nsteps < 0 || !(dt > 0)) return SBP_ERR_INVALID;
  cudaSetDevice(c->d.device);
  // classical RK4 (code/include/time_stepping/time_stepping.h:127-142), a ghost
  // update of each stage input before its stage
  for (long long n = 0; n < nsteps; n++) {
    DCK(halo(c, c->un));
    DCK(stage(c, ST_FIRST, c->un, c->wa, nullptr, dt / 6, 0.5 * dt));
    DCK(halo(c, c->wa));
    DCK(stage(c, ST_MID, c->wa, c->wb, nullptr, dt / 3, 0.5 * dt));
    DCK(halo(c, c->wb));
    DCK(stage(c, ST_MID, c->wb, c->wa, nullptr, dt / 3, dt));
    DCK(halo(c, c->wa));
    DCK(stage(c, ST_LAST, c->wa, nullptr, nullptr, dt / 6, 0.0));
  }
  DCK(cudaStreamSynchronize(c->stream));
  return SBP_OK;
}

}  // extern "C"
