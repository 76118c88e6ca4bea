// wave3d.cuh -- parameters of the 3D acoustic wave stage kernel (wave3d.cu).
//
// The system u_t = -p_x, v_t = -p_y, w_t = -p_z, p_t = -(u_x + v_y + w_z)
// (rho = K = 1) on a box of nx x ny x nz points: the 2D wave_eq_hom system of
// the reference (code/demo/wave_hom/wave_eq_hom_rhs.h) with a third direction,
// which the reference leaves as a TODO (code/include/partitioned_rhs/rhs.h:400-402).
// The same SBP operators act along each axis; the boundary terms are the
// free-surface or the characteristic SAT on all six faces.
//
// State layout: four component planes [u | v | w | p], each nz slabs of ny rows
// of `pitch` elements, so a state is a 2D array of ny*nz rows and every
// row-generic kernel (layout conversion, norms, RK45 combinations) applies.
#pragma once

#include "sbp_device.cuh"

namespace sbp {

template <typename T> struct Wave3Params {
  int nx, ny, nz;
  long long pitch;  // elements per row
  long long slab;   // elements per z slab (ny * pitch)
  long long plane;  // elements per component plane (nz * slab)
  const T* in;      // stage input (4 planes)
  T* un;            // u^n; written in place by ST_LAST
  T* acc;           // RK4 accumulator
  T* wout;          // next stage input
  T* kout;          // ST_RHS output
  T* comp;          // FP32: Kahan compensation of the summed update
  DirTaps<T> dx, dy, dz;  // -hi * stencils per direction
  double bw[3];           // hi * HI[0] per direction: SAT weights (FP64)
  int bc;                 // BC_NONE, BC_FREE_SURFACE or BC_CHARACTERISTIC
  int compensated;        // FP32 state with the Kahan-summed final update
  T c_acc, c_w;           // acc (+)= c_acc * k ; w = u^n + c_w * k
  const int* skip;        // non-null and set: the kernel returns at entry
};

}  // namespace sbp
