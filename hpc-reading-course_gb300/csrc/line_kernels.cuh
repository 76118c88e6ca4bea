// line_kernels.cuh -- fused RHS + SAT + RK4-stage kernels for the scalar
// advection problems (1D and 2D) and the 1D reflection system:
//   advection  u_t = -(a u_x + b u_y)          (code/demo/advection/advection_rhs.h)
//   reflection [u; v]_t = [v_x; u_x]           (code/demo/reflection/reflection_rhs.h)
// One thread per grid point; stencil taps are read through the read-only
// cache (neighbouring threads share them in L1). These problems have 1-2
// components and are a small fraction of the work of the 2D wave system.
#pragma once

#include "sbp_device.cuh"
#include "wave2d.cuh"

namespace sbp {

enum LineKind : int { LK_ADV1D = 0, LK_REFL1D = 1, LK_ADV2D = 2 };

template <typename T> struct LineParams {
  int nx, ny;
  long long pitch, plane;
  const T* in;
  T* un;
  T* acc;
  T* wout;
  T* kout;
  T* comp;
  DirTaps<T> dx, dy;  // advection: -a*hix, -b*hiy scaled (+hix, +hiy with velocity fields); reflection: +hix
  double sat[4];      // advection SAT factors 0.5*tau*hi*HI[0] for W, S, E, N (constant velocities)
  // Advection with a velocity at every point (null: the constants folded into the taps):
  // the velocity planes in T (pitched like the state) for the interior, FP64 copies
  // (nx*ny, row-major) for the SAT, and hi*HI[0] per direction
  const T* va;
  const T* vb;
  const double* va64;
  const double* vb64;
  double bw[2];
  int bc;             // 0: none, 1: the reference's boundary treatment
  int compensated;
  T c_acc, c_w;
  const int* skip;  // non-null and set: the kernel returns at entry
  int* err;
};

// D1 along a line at index i with scaled taps; region choice as rhs_serial.
template <typename T, int ORD>
__device__ __forceinline__ T d1_line(const T* __restrict__ line, long long st, int n, int i, const DirTaps<T>& d) {
  constexpr int W = OpShape<ORD>::W, CS = OpShape<ORD>::CS, R = (W - 1) / 2;
  if (i >= CS && i < n - CS) {
    const T* c = line + (long long)(i - R) * st;
    T s = d.taps[0] * __ldg(c);
#pragma unroll
    for (int k = 1; k < W; k++)
      if (k != R) s = fma(d.taps[k], __ldg(c + k * st), s);
    return s;
  }
  return closure_line<T, ORD>(line, st, n, i, d.cls);
}

// RK4 stage update of one component of one point at offset o.
template <typename T, int STAGE>
__device__ __forceinline__ void line_store(const LineParams<T>& prm, T* wout, const T c_acc, const T c_w, long long o,
                                           T k, T cen) {
  if constexpr (STAGE == ST_RHS) {
    prm.kout[o] = k;
  } else if constexpr (STAGE == ST_FIRST) {
    prm.acc[o] = prm.compensated ? c_acc * k : fma(c_acc, k, cen);
    wout[o] = fma(c_w, k, cen);
  } else if constexpr (STAGE == ST_MID) {
    const T u0 = prm.un[o];
    prm.acc[o] = fma(c_acc, k, prm.acc[o]);
    wout[o] = fma(c_w, k, u0);
  } else {
    const T d = fma(c_acc, k, prm.acc[o]);
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

// SAT_bc_{west,south,east,north} of 2D advection (advection_rhs.h:460-528), FP64,
// at boundary points only (the FP64 round trip is exact elsewhere, and costly on
// the FP64 pipe).
template <typename T>
__device__ __forceinline__ T adv2d_sat(const LineParams<T>& prm, int i, int j, T k, T cen) {
  if (prm.bc && (i == 0 || j == 0 || i == prm.nx - 1 || j == prm.ny - 1)) {
    double kk = (double)k;
    const double u = (double)cen;
    if (prm.va64) {  // tau from the velocity at the boundary point
      const long long g = (long long)j * prm.nx + i;
      const double a = prm.va64[g], b = prm.vb64[g];
      if (i == 0) kk += 0.5 * (-0.5 * (a + fabs(a))) * prm.bw[0] * u;
      if (j == 0) kk += 0.5 * (-0.5 * (b + fabs(b))) * prm.bw[1] * u;
      if (i == prm.nx - 1) kk += 0.5 * (0.5 * (a - fabs(a))) * prm.bw[0] * u;
      if (j == prm.ny - 1) kk += 0.5 * (0.5 * (b - fabs(b))) * prm.bw[1] * u;
      return (T)kk;
    }
    if (i == 0) kk += prm.sat[0] * u;
    if (j == 0) kk += prm.sat[1] * u;
    if (i == prm.nx - 1) kk += prm.sat[2] * u;
    if (j == prm.ny - 1) kk += prm.sat[3] * u;
    return (T)kk;
  }
  return k;
}

// One grid point of a stage: RHS, boundary terms and the RK4 stage update.
template <typename T, int ORD, int KIND, int STAGE>
__device__ __forceinline__ void line_point(const LineParams<T>& prm, const T* __restrict__ in, T* wout, const T c_acc,
                                           const T c_w, const int i, const int j) {
  const int nx = prm.nx, ny = prm.ny;
  const long long pitch = prm.pitch, plane = prm.plane;
  const long long q = (long long)j * pitch + i;
  constexpr int NC = (KIND == LK_REFL1D) ? 2 : 1;
  T k[NC];
  T cen[NC];
  if constexpr (KIND == LK_ADV1D) {
    k[0] = d1_line<T, ORD>(in, 1, nx, i, prm.dx);
    if (prm.va) k[0] = -prm.va[q] * k[0];  // -a(i) D1 u
    cen[0] = in[q];
    if (prm.bc) {  // SAT_bc_l / SAT_bc_r (advection_rhs.h:94-119)
      if (prm.va64) {
        if (i == 0 || i == nx - 1) {
          const double a = prm.va64[i];
          const double tau = i == 0 ? -0.5 * (a + fabs(a)) : 0.5 * (a - fabs(a));
          k[0] = (T)((double)k[0] + 0.5 * tau * prm.bw[0] * (double)cen[0]);
        }
      } else {
        if (i == 0) k[0] = (T)((double)k[0] + prm.sat[0] * (double)cen[0]);
        if (i == nx - 1) k[0] = (T)((double)k[0] + prm.sat[2] * (double)cen[0]);
      }
    }
  } else if constexpr (KIND == LK_ADV2D) {
    const T* row = in + (long long)j * pitch;
    const T* col = in + i;
    if (prm.va) {  // -(a(i,j) D1x u + b(i,j) D1y u)
      k[0] = -(prm.va[q] * d1_line<T, ORD>(row, 1, nx, i, prm.dx) + prm.vb[q] * d1_line<T, ORD>(col, pitch, ny, j, prm.dy));
    } else {
      k[0] = d1_line<T, ORD>(row, 1, nx, i, prm.dx) + d1_line<T, ORD>(col, pitch, ny, j, prm.dy);
    }
    cen[0] = in[q];
    k[0] = adv2d_sat<T>(prm, i, j, k[0], cen[0]);
  } else {  // LK_REFL1D: dst(i,1) = D1 u, dst(i,0) = D1 v
    k[1] = d1_line<T, ORD>(in, 1, nx, i, prm.dx);
    k[0] = d1_line<T, ORD>(in + plane, 1, nx, i, prm.dx);
    cen[0] = in[q];
    cen[1] = in[plane + q];
    if (prm.bc && (i == 0 || i == nx - 1)) k[0] = T(0);  // proj_dirichlet_bc_{l,r}
  }
#pragma unroll
  for (int c = 0; c < NC; c++) line_store<T, STAGE>(prm, wout, c_acc, c_w, c * plane + q, k[c], cen[c]);
}

template <typename T, int ORD, int KIND, int STAGE>
__global__ void __launch_bounds__(256) line_stage_kernel(const __grid_constant__ LineParams<T> prm) {
  if (prm.skip && *prm.skip) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= prm.nx || j >= prm.ny) return;
  line_point<T, ORD, KIND, STAGE>(prm, prm.in, prm.wout, prm.c_acc, prm.c_w, i, j);
}

}  // namespace sbp
