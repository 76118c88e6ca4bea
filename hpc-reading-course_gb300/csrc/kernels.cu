// kernels.cu -- launchers for the scalar/1D stage kernels, the AoS <-> SoA
// layout kernels at the reference boundary, the FP64 norm reductions and the
// FP64 throughput probe.
#include "launch.h"

namespace sbp {

int wave_smem_bytes(int order, bool fp32) {
  switch (order) {
    case 2: return fp32 ? WaveStageTile<float, 2, WK_HOM, ST_MID>::SMEM : WaveStageTile<double, 2, WK_HOM, ST_MID>::SMEM;
    case 4: return fp32 ? WaveStageTile<float, 4, WK_HOM, ST_MID>::SMEM : WaveStageTile<double, 4, WK_HOM, ST_MID>::SMEM;
    case 6: return fp32 ? WaveStageTile<float, 6, WK_HOM, ST_MID>::SMEM : WaveStageTile<double, 6, WK_HOM, ST_MID>::SMEM;
    default: return -1;
  }
}

int device_sm_count() {
  static int cache[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 148;
  if (dev < 64 && cache[dev]) return cache[dev];
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
  if (dev < 64) cache[dev] = n;
  return n;
}

// ---------------------------------------------------------------- line kernels
namespace {
template <typename T, int ORD, int KIND>
cudaError_t line_stage(int stage, const LineParams<T>& prm, cudaStream_t s) {
  const dim3 block(KIND == LK_ADV2D ? 32 : 128, KIND == LK_ADV2D ? 8 : 1);
  const dim3 grid((prm.nx + block.x - 1) / block.x, (prm.ny + block.y - 1) / block.y);
  switch (stage) {
    case ST_RHS: line_stage_kernel<T, ORD, KIND, ST_RHS><<<grid, block, 0, s>>>(prm); break;
    case ST_FIRST: line_stage_kernel<T, ORD, KIND, ST_FIRST><<<grid, block, 0, s>>>(prm); break;
    case ST_MID: line_stage_kernel<T, ORD, KIND, ST_MID><<<grid, block, 0, s>>>(prm); break;
    case ST_LAST: line_stage_kernel<T, ORD, KIND, ST_LAST><<<grid, block, 0, s>>>(prm); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <typename T, int ORD>
cudaError_t line_order(int kind, int stage, const LineParams<T>& prm, cudaStream_t s) {
  switch (kind) {
    case LK_ADV1D: return line_stage<T, ORD, LK_ADV1D>(stage, prm, s);
    case LK_REFL1D: return line_stage<T, ORD, LK_REFL1D>(stage, prm, s);
    case LK_ADV2D: return line_stage<T, ORD, LK_ADV2D>(stage, prm, s);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace

template <typename T>
cudaError_t launch_line(int order, int kind, int stage, const LineParams<T>& prm, cudaStream_t s) {
  switch (order) {
    case 2: return line_order<T, 2>(kind, stage, prm, s);
    case 4: return line_order<T, 4>(kind, stage, prm, s);
    case 6: return line_order<T, 6>(kind, stage, prm, s);
    default: return cudaErrorInvalidValue;
  }
}
template cudaError_t launch_line<double>(int, int, int, const LineParams<double>&, cudaStream_t);
template cudaError_t launch_line<float>(int, int, int, const LineParams<float>&, cudaStream_t);

// ---------------------------------------------------------------- layout
// One thread per (point, component) of the AoS array: reads are contiguous,
// writes go to `dofs` planes (contiguous per component within a warp).
template <typename T>
__global__ void pack_kernel(const double* __restrict__ aos, T* __restrict__ soa, int nx, int ny, int dofs,
                            long long pitch, long long plane) {
  const long long n = (long long)nx * ny * dofs;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long pt = e / dofs;
    const int c = (int)(e - pt * dofs);
    const long long j = pt / nx, i = pt - j * nx;
    soa[c * plane + j * pitch + i] = (T)aos[e];
  }
}

template <typename T>
__global__ void unpack_kernel(const T* __restrict__ soa, double* __restrict__ aos, int nx, int ny, int dofs,
                              long long pitch, long long plane) {
  const long long n = (long long)nx * ny * dofs;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long pt = e / dofs;
    const int c = (int)(e - pt * dofs);
    const long long j = pt / nx, i = pt - j * nx;
    aos[e] = (double)soa[c * plane + j * pitch + i];
  }
}

static int grid_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  if (b > 152LL * 16) b = 152LL * 16;
  return (int)(b < 1 ? 1 : b);
}

template <typename T>
cudaError_t launch_pack(const double* aos, T* soa, int nx, int ny, int dofs, long long pitch, long long plane,
                        cudaStream_t s) {
  const long long n = (long long)nx * ny * dofs;
  pack_kernel<T><<<grid_for(n, 256), 256, 0, s>>>(aos, soa, nx, ny, dofs, pitch, plane);
  return cudaGetLastError();
}
template <typename T>
cudaError_t launch_unpack(const T* soa, double* aos, int nx, int ny, int dofs, long long pitch, long long plane,
                          cudaStream_t s) {
  const long long n = (long long)nx * ny * dofs;
  unpack_kernel<T><<<grid_for(n, 256), 256, 0, s>>>(soa, aos, nx, ny, dofs, pitch, plane);
  return cudaGetLastError();
}
template cudaError_t launch_pack<double>(const double*, double*, int, int, int, long long, long long, cudaStream_t);
template cudaError_t launch_pack<float>(const double*, float*, int, int, int, long long, long long, cudaStream_t);
template cudaError_t launch_unpack<double>(const double*, double*, int, int, int, long long, long long, cudaStream_t);
template cudaError_t launch_unpack<float>(const float*, double*, int, int, int, long long, long long, cudaStream_t);

// ---------------------------------------------------------------- reductions
// Two passes with a fixed block count, so the summation order (and the FP64
// result) does not depend on timing.
constexpr int kReduceThreads = 256;

__device__ __forceinline__ void block_reduce2(double& sum, double& mx, double* sh) {
  for (int o = 16; o > 0; o >>= 1) {
    sum += __shfl_down_sync(0xffffffffu, sum, o);
    mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sh[warp] = sum;
    sh[32 + warp] = mx;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    sum = lane < nw ? sh[lane] : 0.0;
    mx = lane < nw ? sh[32 + lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      sum += __shfl_down_sync(0xffffffffu, sum, o);
      mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads)
    error_partial_kernel(const T* __restrict__ soa, const double* __restrict__ aos, int nx, int ny, int dofs,
                         long long pitch, long long plane, double* __restrict__ partial) {
  __shared__ double sh[64];
  double sum = 0.0, mx = 0.0;
  const long long n = (long long)nx * ny * dofs;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long pt = e / dofs;
    const int c = (int)(e - pt * dofs);
    const long long j = pt / nx, i = pt - j * nx;
    const double d = fabs(aos[e] - (double)soa[c * plane + j * pitch + i]);
    sum += d * d;
    mx = fmax(mx, d);
  }
  block_reduce2(sum, mx, sh);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = sum;
    partial[2 * blockIdx.x + 1] = mx;
  }
}

__global__ void __launch_bounds__(kReduceThreads) final_reduce_kernel(const double* __restrict__ partial, int nblocks,
                                                                      double* __restrict__ out) {
  __shared__ double sh[64];
  double sum = 0.0, mx = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    sum += partial[2 * b];
    mx = fmax(mx, partial[2 * b + 1]);
  }
  block_reduce2(sum, mx, sh);
  if (threadIdx.x == 0) {
    out[0] = sum;
    out[1] = mx;
  }
}

template <typename T>
cudaError_t launch_error_norms(const T* soa, const double* aos, int nx, int ny, int dofs, long long pitch,
                               long long plane, double* partial, double* out, cudaStream_t s) {
  error_partial_kernel<T><<<kReduceBlocks, kReduceThreads, 0, s>>>(soa, aos, nx, ny, dofs, pitch, plane, partial);
  final_reduce_kernel<<<1, kReduceThreads, 0, s>>>(partial, kReduceBlocks, out);
  return cudaGetLastError();
}
template cudaError_t launch_error_norms<double>(const double*, const double*, int, int, int, long long, long long,
                                                double*, double*, cudaStream_t);
template cudaError_t launch_error_norms<float>(const float*, const double*, int, int, int, long long, long long,
                                               double*, double*, cudaStream_t);

// Quadrature weights of the closures (code/include/sbpops/H_central.h:193-212).
__constant__ double c_hquad[3][6] = {
    {1. / 2, 0, 0, 0, 0, 0},
    {17. / 48, 59. / 48, 43. / 48, 49. / 48, 0, 0},
    {13649. / 43200, 12013. / 8640, 2711. / 4320, 5359. / 4320, 7877. / 8640, 43801. / 43200}};

__device__ __forceinline__ double hweight(int n, int i, int cs, int oi) {
  if (i < cs) return c_hquad[oi][i];
  if (i >= n - cs) return c_hquad[oi][n - 1 - i];
  return 1.0;
}

template <typename T>
__global__ void __launch_bounds__(kReduceThreads)
    hnorm_partial_kernel(const T* __restrict__ soa, int nx, int ny, int dofs, long long pitch, long long plane,
                         int order, double hx, double hy, int ysplit, double* __restrict__ partial, int nz,
                         double hz) {
  __shared__ double sh[64];
  const int oi = order / 2 - 1, cs = (order == 2) ? 1 : (order == 4 ? 4 : 6);
  double sum = 0.0, mx = 0.0;
  const long long n = (long long)nx * ny * nz;
  for (long long pt = blockIdx.x * (long long)blockDim.x + threadIdx.x; pt < n; pt += (long long)gridDim.x * blockDim.x) {
    const long long r = pt / nx, i = pt - r * nx;  // row r = j + ny * k
    const long long kz = r / ny, j = r - kz * ny;
    // two-block grids: each block has its own quadrature in y
    const int jb0 = (ysplit > 0 && j >= ysplit) ? ysplit : 0;
    const int nyb = (ysplit > 0) ? (j >= ysplit ? ny - ysplit : ysplit) : ny;
    double w = hx * hweight(nx, (int)i, cs, oi) * (ny > 1 ? hy * hweight(nyb, (int)j - jb0, cs, oi) : 1.0);
    if (nz > 1) w *= hz * hweight(nz, (int)kz, cs, oi);
    double s = 0.0;
    for (int c = 0; c < dofs; c++) {
      const double x = (double)soa[c * plane + r * pitch + i];
      s += x * x;
    }
    sum += w * s;
  }
  block_reduce2(sum, mx, sh);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = sum;
    partial[2 * blockIdx.x + 1] = 0.0;
  }
}

template <typename T>
cudaError_t launch_hnorm(const T* soa, int nx, int ny, int dofs, long long pitch, long long plane, int order,
                         double hx, double hy, int ysplit, double* partial, double* out, cudaStream_t s, int nz,
                         double hz) {
  hnorm_partial_kernel<T><<<kReduceBlocks, kReduceThreads, 0, s>>>(soa, nx, ny, dofs, pitch, plane, order, hx, hy,
                                                                   ysplit, partial, nz, hz);
  final_reduce_kernel<<<1, kReduceThreads, 0, s>>>(partial, kReduceBlocks, out);
  return cudaGetLastError();
}
template cudaError_t launch_hnorm<double>(const double*, int, int, int, long long, long long, int, double, double,
                                          int, double*, double*, cudaStream_t, int, double);
template cudaError_t launch_hnorm<float>(const float*, int, int, int, long long, long long, int, double, double, int,
                                         double*, double*, cudaStream_t, int, double);

// ---------------------------------------------------------------- FP64 probe
__global__ void dfma_probe_kernel(double* out, int iters) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = 1.0 + 1e-9 * (threadIdx.x + k);
  const double m = 0.9999999, c = 1e-7;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = fma(a[k], m, c);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += a[k];
  if (s == 12345.678) out[0] = s;  // keeps the chains live; never true in practice
  if (threadIdx.x == 0 && blockIdx.x == 0) out[1] = s;
}

cudaError_t launch_dfma_probe(double* out, int blocks, int threads, int iters, cudaStream_t s) {
  dfma_probe_kernel<<<blocks, threads, 0, s>>>(out, iters);
  return cudaGetLastError();
}

}  // namespace sbp
