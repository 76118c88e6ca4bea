// rk45.cu -- adaptive Runge-Kutta-Fehlberg 4(5) on the device-resident state.
//
// Replaces the reference's ts_rk45 (code/src/time_stepping/ts_rk.cpp:41-52),
// which hands the RHS callback to PETSc's TSRK5F (Fehlberg 4(5), the step is
// advanced with the 5th-order weights) under TSADAPTBASIC with
// TS_EXACTFINALTIME_MATCHSTEP. PETSc is not part of the reference and its
// version is not pinned; the tableau is Fehlberg's published one and the
// controller restates PETSc's documented basic adaptor (see rk45_control_kernel).
//
// One attempted step is a fixed kernel sequence, so that a chunk of attempts
// is captured once as a CUDA graph and replayed without host round trips:
//   RHS(u) -> k1, combine -> w, RHS(w) -> k2, ..., RHS(w) -> k6,
//   final (u5, error partial sums), control (1 block), accept copy.
// Step size, time and the stop flag live in device memory (Rk45Ctrl); after the
// run stops every kernel of the remaining attempts returns at entry.
#include <cuda_runtime.h>

#include <cmath>

#include "launch.h"
#include "rkf_tableau.cuh"

namespace sbp {

constexpr int kRkfThreads = 256;

// Row r of the SoA state (component c = r / ny, grid row j = r % ny) starts at
// c * plane + j * pitch and holds nx valid points.
__device__ __forceinline__ long long rkf_row(int r, int ny, long long pitch, long long plane) {
  const int c = r / ny, j = r - c * ny;
  return (long long)c * plane + (long long)j * pitch;
}

// w = u + h * (sum_{j<S} a[S][j] k_j), the input of stage S+1 (S = 1..5); the sum
// runs left to right with fused multiply-adds.
template <int S>
__global__ void __launch_bounds__(kRkfThreads) rkf_combine_kernel(Rk45Buffers b, const Rk45Ctrl* __restrict__ ctrl) {
  if (ctrl->done) return;
  const double h = ctrl->h;
  const int rows = b.dofs * b.ny;
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const long long o0 = rkf_row(r, b.ny, b.pitch, b.plane);
    for (int i = threadIdx.x; i < b.nx; i += blockDim.x) {
      const long long o = o0 + i;
      double s = kRkfA[S][0] * b.k[0][o];
#pragma unroll
      for (int j = 1; j < S; j++) s = fma(kRkfA[S][j], b.k[j][o], s);
      b.w[o] = fma(h, s, b.u[o]);
    }
  }
}

// u5 = u + h * sum b5_j k_j (written to unew), u4 = u + h * sum b4_j k_j, and the
// per-block partial sum of ((u5 - u4) / (atol + rtol * max(|u5|, |u4|)))^2
// (rkf_candidate, rkf_err_term).
__global__ void __launch_bounds__(kRkfThreads) rkf_final_kernel(Rk45Buffers b, Rk45Ctrl* __restrict__ ctrl) {
  __shared__ double red[kRkfThreads];
  if (ctrl->done) return;
  const double h = ctrl->h, atol = ctrl->atol, rtol = ctrl->rtol;
  const int rows = b.dofs * b.ny;
  double acc = 0.0;
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const long long o0 = rkf_row(r, b.ny, b.pitch, b.plane);
    for (int i = threadIdx.x; i < b.nx; i += blockDim.x) {
      const long long o = o0 + i;
      double u5, u4;
      rkf_candidate(b.u[o], h, b.k[0][o], b.k[2][o], b.k[3][o], b.k[4][o], b.k[5][o], u5, u4);
      b.unew[o] = u5;
      acc += rkf_err_term(u5, u4, atol, rtol);
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kRkfThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) b.partial[blockIdx.x] = red[0];
}

// The step-size controller, restating PETSc's TSADAPTBASIC with
// TS_EXACTFINALTIME_MATCHSTEP (one thread decides; the block sums the partials
// in a fixed order first):
//   wlte = sqrt(sum / n)                         weighted RMS error (2-norm form)
//   accept iff wlte <= 1 (or h is at dt_min)
//   safety' = safety * reject_safety if this and the previous attempt failed
//   h' = h * clip(safety' * wlte^(-1/5), clip_lo, clip_hi), then into [dt_min, dt_max]
//   landing on t_end: with hmax = t_end - t, h' > hmax -> hmax; otherwise
//   2 h' > hmax -> hmax / 2, and 1.01 h' > hmax -> hmax.
// Stops when the step that lands on t_end is accepted, after max_reject
// rejections in a row, after max_steps attempts, or on a non-finite error.
__global__ void __launch_bounds__(kRkfThreads) rkf_control_kernel(const double* __restrict__ partial, int nparts,
                                                                  Rk45Ctrl* __restrict__ ctrl) {
  __shared__ double red[kRkfThreads];
  Rk45Ctrl& c = *ctrl;
  if (c.done) {
    if (threadIdx.x == 0) c.copy_pending = 0;
    return;
  }
  double s = 0.0;
  for (int p = threadIdx.x; p < nparts; p += blockDim.x) s += partial[p];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int k = kRkfThreads / 2; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  const double wlte = sqrt(red[0] / c.n);
  c.wlte = wlte;
  const double h = c.h;
  if (!(wlte <= 1e300)) {  // NaN or infinite: stop without taking the step
    c.copy_pending = 0;
    c.done = 1;
    c.status = RK45_NONFINITE;
    c.rejected++;
    return;
  }
  double safety = c.safety;
  bool accept = true;
  if (wlte > 1.0) {
    if (!c.last_accepted) safety *= c.reject_safety;
    accept = h < (1.0 + 1.4901161193847656e-08) * c.dt_min;
  }
  double hfac = wlte > 0.0 ? safety * pow(wlte, -0.2) : c.clip_hi;
  hfac = fmin(fmax(hfac, c.clip_lo), c.clip_hi);
  double hn = fmin(fmax(h * hfac, c.dt_min), c.dt_max);
  c.copy_pending = accept ? 1 : 0;
  c.last_accepted = accept ? 1 : 0;
  if (accept) {
    c.accepted++;
    c.rejects_in_row = 0;
    if (c.final_step) {
      c.t = c.t_end;
      c.done = 1;
      c.status = RK45_OK;
      c.h = hn;
      return;
    }
    c.t = c.t + h;
  } else {
    c.rejected++;
    c.rejects_in_row++;
  }
  const double hmax = c.t_end - c.t;
  const double h0 = hn;
  int fin = 0;
  if (h0 >= hmax) {
    hn = hmax;
    fin = 1;
  } else {
    if (2.0 * h0 > hmax) hn = 0.5 * hmax;
    if (1.01 * h0 > hmax) {
      hn = hmax;
      fin = 1;
    }
  }
  c.h = hn;
  c.final_step = fin;
  if (c.rejects_in_row >= c.max_reject) {
    c.done = 1;
    c.status = RK45_REJECTED;
  } else if (c.accepted + c.rejected >= c.max_steps) {
    c.done = 1;
    c.status = RK45_STEP_LIMIT;
  }
}

// u = unew after an accepted attempt (whole planes, padding included).
__global__ void __launch_bounds__(kRkfThreads) rkf_accept_kernel(Rk45Buffers b, const Rk45Ctrl* __restrict__ ctrl) {
  if (!ctrl->copy_pending) return;
  const long long n = (long long)b.dofs * b.plane;
  const double2* src = reinterpret_cast<const double2*>(b.unew);
  double2* dst = reinterpret_cast<double2*>(b.u);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n / 2; e += (long long)gridDim.x * blockDim.x)
    dst[e] = src[e];
}

cudaError_t launch_rk45_combine(int stage, const Rk45Buffers& b, const Rk45Ctrl* ctrl, cudaStream_t s) {
  const int rows = b.dofs * b.ny;
  const unsigned grid = (unsigned)(rows < kReduceBlocks ? rows : kReduceBlocks);
  switch (stage) {
    case 1: rkf_combine_kernel<1><<<grid, kRkfThreads, 0, s>>>(b, ctrl); break;
    case 2: rkf_combine_kernel<2><<<grid, kRkfThreads, 0, s>>>(b, ctrl); break;
    case 3: rkf_combine_kernel<3><<<grid, kRkfThreads, 0, s>>>(b, ctrl); break;
    case 4: rkf_combine_kernel<4><<<grid, kRkfThreads, 0, s>>>(b, ctrl); break;
    case 5: rkf_combine_kernel<5><<<grid, kRkfThreads, 0, s>>>(b, ctrl); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_rk45_finish(const Rk45Buffers& b, Rk45Ctrl* ctrl, cudaStream_t s) {
  // the partial-sum count is fixed (kReduceBlocks) so the sum order is the same every attempt
  rkf_final_kernel<<<kReduceBlocks, kRkfThreads, 0, s>>>(b, ctrl);
  return launch_rk45_control(b, kReduceBlocks, ctrl, s);
}

cudaError_t launch_rk45_control(const Rk45Buffers& b, int nparts, Rk45Ctrl* ctrl, cudaStream_t s) {
  rkf_control_kernel<<<1, kRkfThreads, 0, s>>>(b.partial, nparts, ctrl);
  rkf_accept_kernel<<<kReduceBlocks, kRkfThreads, 0, s>>>(b, ctrl);
  return cudaGetLastError();
}

}  // namespace sbp
