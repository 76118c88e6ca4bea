// wave3d.cu -- fused RHS + SAT + RK4-stage kernel of the 3D acoustic wave
// system (wave3d.cuh), orders 2, 4 and 6, FP64 or compensated FP32.
//
// One thread per (i, j) column of a 64 x 4 block, marching 16 z planes. In FP64
// the kernel is bound by the FP64 pipe (about 31 FP64 instructions per point and
// stage against 128-160 bytes of state traffic), so the stencil taps are plain
// read-only loads: neighbours along x share cache lines within a warp, along y
// within the block, and along z the thread re-reads the planes it touched last.
#include <cuda_runtime.h>

#include "launch.h"

namespace sbp {

constexpr int kW3X = 64, kW3Y = 4, kW3Z = 16;

// Boundary terms on the faces the point lies on (FP64 arithmetic, as the 2D kernels):
// free surface (wave_eq_hom_rhs.h:389-441 per face): lower face F_ud -= bw_d p, upper F_ud += bw_d p;
// characteristic (Z = c = 1): lower face g = bw_d (p + u_d): F_ud -= g/2, F_p -= g/2;
// upper face g = bw_d (p - u_d): F_ud += g/2, F_p -= g/2.
template <typename T> struct Rhs4 { T u, v, w, p; };

template <typename T>
__device__ __noinline__ Rhs4<T> wave3d_sat(const Wave3Params<T>& prm, int i, int j, int k, T uc, T vc, T wc, T pc,
                                           Rhs4<T> kc) {
  // values and results by value: a noinline function taking arrays by reference
  // would keep the caller's arrays in local memory on every point
  double f[4] = {(double)kc.u, (double)kc.v, (double)kc.w, (double)kc.p};
  const double cen[3] = {(double)uc, (double)vc, (double)wc};
  const int idx[3] = {i, j, k};
  const int n[3] = {prm.nx, prm.ny, prm.nz};
  const double p = (double)pc;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const bool lo = idx[d] == 0, hi = idx[d] == n[d] - 1;
    if (!lo && !hi) continue;
    const double ud = cen[d];
    if (prm.bc == BC_CHARACTERISTIC) {
      if (lo) {
        const double g = prm.bw[d] * (p + ud);
        f[d] -= 0.5 * g;
        f[3] -= 0.5 * g;
      }
      if (hi) {
        const double g = prm.bw[d] * (p - ud);
        f[d] += 0.5 * g;
        f[3] -= 0.5 * g;
      }
    } else {
      if (lo) f[d] -= prm.bw[d] * p;
      if (hi) f[d] += prm.bw[d] * p;
    }
  }
  return Rhs4<T>{(T)f[0], (T)f[1], (T)f[2], (T)f[3]};
}

// FP64: the z neighbours of p and w come from a per-thread register window (one new
// value of each per plane instead of the five taps); measured at 256^3, order 4:
// 1.209e10 against 1.170e10 point-stages/s. FP32 runs faster without it (3.48e10
// against 3.25e10: at its 40-register budget the window spills).
template <typename T> constexpr bool w3_zwin() { return sizeof(T) == 8; }

// Interior D1 over W values of a register window, in d1_line's order.
template <typename T, int ORD>
__device__ __forceinline__ T taps_window(const DirTaps<T>& d, const T (&c)[OpShape<ORD>::W]) {
  constexpr int W = OpShape<ORD>::W, R = (W - 1) / 2;
  T s = d.taps[0] * c[0];
#pragma unroll
  for (int q = 1; q < W; q++)
    if (q != R) s = fma(d.taps[q], c[q], s);
  return s;
}

template <typename T, int ORD, int STAGE>
__device__ __forceinline__ void wave3d_point(const Wave3Params<T>& prm, int i, int j, int k,
                                             const T (&pw)[OpShape<ORD>::W], const T (&ww)[OpShape<ORD>::W]) {
  const int nx = prm.nx, ny = prm.ny, nz = prm.nz;
  const long long pitch = prm.pitch, slab = prm.slab, plane = prm.plane;
  const T* __restrict__ U = prm.in;
  const T* __restrict__ V = U + plane;
  const T* __restrict__ W = V + plane;
  const T* __restrict__ P = W + plane;
  const long long xo = (long long)k * slab + (long long)j * pitch;  // start of the x line
  const long long yo = (long long)k * slab + i;                     // start of the y line (stride pitch)
  const long long zo = (long long)j * pitch + i;                    // start of the z line (stride slab)
  const long long q = xo + i;
  T kc[4];
  kc[0] = d1_line<T, ORD>(P + xo, 1, nx, i, prm.dx);
  kc[1] = d1_line<T, ORD>(P + yo, pitch, ny, j, prm.dy);
  constexpr int CS = OpShape<ORD>::CS;
  const bool zwin = w3_zwin<T>() && k >= CS && k < nz - CS;
  kc[2] = zwin ? taps_window<T, ORD>(prm.dz, pw) : d1_line<T, ORD>(P + zo, slab, nz, k, prm.dz);
  kc[3] = d1_line<T, ORD>(U + xo, 1, nx, i, prm.dx) + d1_line<T, ORD>(V + yo, pitch, ny, j, prm.dy) +
          (zwin ? taps_window<T, ORD>(prm.dz, ww) : d1_line<T, ORD>(W + zo, slab, nz, k, prm.dz));
  const T cen[4] = {__ldg(U + q), __ldg(V + q), __ldg(W + q), __ldg(P + q)};
  if (prm.bc != BC_NONE && (i == 0 || j == 0 || k == 0 || i == nx - 1 || j == ny - 1 || k == nz - 1)) {
    const Rhs4<T> r = wave3d_sat<T>(prm, i, j, k, cen[0], cen[1], cen[2], cen[3], Rhs4<T>{kc[0], kc[1], kc[2], kc[3]});
    kc[0] = r.u;
    kc[1] = r.v;
    kc[2] = r.w;
    kc[3] = r.p;
  }
  // RK4 stage update (classical RK4, code/include/time_stepping/time_stepping.h:127-142)
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const long long o = c * plane + q;
    if constexpr (STAGE == ST_RHS) {
      prm.kout[o] = kc[c];
    } else if constexpr (STAGE == ST_FIRST) {
      st_stream(prm.acc + o, prm.compensated ? prm.c_acc * kc[c] : fma(prm.c_acc, kc[c], cen[c]));
      st_stream(prm.wout + o, fma(prm.c_w, kc[c], cen[c]));
    } else if constexpr (STAGE == ST_MID) {
      st_stream(prm.acc + o, fma(prm.c_acc, kc[c], prm.acc[o]));
      st_stream(prm.wout + o, fma(prm.c_w, kc[c], prm.un[o]));
    } else {  // ST_LAST
      const T d = fma(prm.c_acc, kc[c], prm.acc[o]);
      if (prm.compensated) {
        const T u0 = prm.un[o], e = prm.comp[o];
        const T yv = d - e;
        const T tv = u0 + yv;
        prm.comp[o] = (tv - u0) - yv;
        prm.un[o] = tv;
      } else {
        prm.un[o] = d;
      }
    }
  }
}

// Blocks per SM the register budget is sized for: the kernel is latency-bound, so
// occupancy pays (measured at 256^3, order 4: FP64 1.02e10 / 1.14e10 / 1.17e10
// point-stages/s at 2 / 3 / 4 blocks, flat beyond; FP32 1.48e10 / 2.10e10 /
// 2.67e10 / 3.07e10 / 3.48e10 at 2 .. 6).
#ifndef SBP_W3_BLOCKS_F64
#define SBP_W3_BLOCKS_F64 4
#endif
#ifndef SBP_W3_BLOCKS_F32
#define SBP_W3_BLOCKS_F32 6
#endif
template <typename T, int ORD, int STAGE>
__global__ void __launch_bounds__(kW3X * kW3Y, sizeof(T) == 8 ? SBP_W3_BLOCKS_F64 : SBP_W3_BLOCKS_F32)
    wave3d_stage_kernel(const __grid_constant__ Wave3Params<T> prm) {
  if (prm.skip && *prm.skip) return;
  const int i = blockIdx.x * kW3X + threadIdx.x;
  const int j = blockIdx.y * kW3Y + threadIdx.y;
  if (i >= prm.nx || j >= prm.ny) return;
  const int k0 = blockIdx.z * kW3Z;
  const int k1 = k0 + kW3Z < prm.nz ? k0 + kW3Z : prm.nz;
  constexpr int W = OpShape<ORD>::W, R = (W - 1) / 2;
  T pw[W], ww[W];  // p and w at planes k - R .. k + R of this column (zero outside the grid)
  const long long zo = (long long)j * prm.pitch + i;
  const T* Pz = prm.in + 3 * prm.plane + zo;
  const T* Wz = prm.in + 2 * prm.plane + zo;
  if constexpr (w3_zwin<T>()) {
#pragma unroll
    for (int s = 0; s < W; s++) {
      const int kk = k0 - R + s;
      const bool in = kk >= 0 && kk < prm.nz;
      pw[s] = in ? __ldg(Pz + kk * prm.slab) : T(0);
      ww[s] = in ? __ldg(Wz + kk * prm.slab) : T(0);
    }
  }
#pragma unroll 1
  for (int k = k0; k < k1; k++) {
    T pn = T(0), wn = T(0);
    const int kn = k + 1 + R;
    if (w3_zwin<T>() && kn < prm.nz && k + 1 < k1) {  // the window's next plane, loaded ahead
      pn = __ldg(Pz + kn * prm.slab);
      wn = __ldg(Wz + kn * prm.slab);
    }
    wave3d_point<T, ORD, STAGE>(prm, i, j, k, pw, ww);
    if constexpr (w3_zwin<T>()) {
#pragma unroll
      for (int s = 0; s + 1 < W; s++) {
        pw[s] = pw[s + 1];
        ww[s] = ww[s + 1];
      }
      pw[W - 1] = pn;
      ww[W - 1] = wn;
    }
  }
}

namespace {

template <typename T, int ORD>
cudaError_t wave3d_order(int stage, const Wave3Params<T>& prm, cudaStream_t s) {
  const dim3 block(kW3X, kW3Y);
  const dim3 grid((prm.nx + kW3X - 1) / kW3X, (prm.ny + kW3Y - 1) / kW3Y, (prm.nz + kW3Z - 1) / kW3Z);
  switch (stage) {
    case ST_RHS: wave3d_stage_kernel<T, ORD, ST_RHS><<<grid, block, 0, s>>>(prm); break;
    case ST_FIRST: wave3d_stage_kernel<T, ORD, ST_FIRST><<<grid, block, 0, s>>>(prm); break;
    case ST_MID: wave3d_stage_kernel<T, ORD, ST_MID><<<grid, block, 0, s>>>(prm); break;
    case ST_LAST: wave3d_stage_kernel<T, ORD, ST_LAST><<<grid, block, 0, s>>>(prm); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t launch_wave3d(int order, int stage, const Wave3Params<T>& prm, cudaStream_t s) {
  if (prm.nz > 65535 * kW3Z || prm.ny > 65535 * kW3Y) return cudaErrorInvalidValue;
  switch (order) {
    case 2: return wave3d_order<T, 2>(stage, prm, s);
    case 4: return wave3d_order<T, 4>(stage, prm, s);
    case 6: return wave3d_order<T, 6>(stage, prm, s);
    default: return cudaErrorInvalidValue;
  }
}
template cudaError_t launch_wave3d<double>(int, int, const Wave3Params<double>&, cudaStream_t);
template cudaError_t launch_wave3d<float>(int, int, const Wave3Params<float>&, cudaStream_t);

}  // namespace sbp
