// launch.h -- host-side launchers for the SBP kernels (implemented in the .cu
// files of this directory, one translation unit per operator order for the
// 2D wave kernels so they compile in parallel).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "line_kernels.cuh"
#include "wave2d.cuh"
#include "wave3d.cuh"
#include "wave_batch.cuh"

namespace sbp {

struct WaveMaps {
  CUtensorMap p, u, v;  // the stage input seen with the p, u and v tile boxes (with halos)
  CUtensorMap n, a, c;  // u^n, acc and the FP32 Kahan term as 3-component point boxes
  CUtensorMap k;        // variable coefficients [1/rho | K] as a 2-component point box
};

// Tile height of the single-instance wave stage kernel (see wave_ty).
inline int wave_tile_height(int elem_bytes, int kind = WK_HOM) {
  if (elem_bytes == 8) return kind == WK_HOM ? wave_ty<double, WK_HOM>() : wave_ty<double, WK_VAR>();
  return kind == WK_VAR ? wave_ty<float, WK_VAR>() : wave_ty<float, WK_HOM>();
}

// Scales of the fixed-point FP64 stages (wave2d_fixed.cuh) for one launch: the
// RHS in units of sigma = -hi/den per direction, and the stage's RK4
// coefficients times sigma of each component (u and p: x, v: y). Every launch of
// a constant-coefficient FP64 stage sets them; the kernel refuses to run without.
inline void set_fixed_scales(WaveParams<double>& p, int order, double hix, double hiy) {
  const double den = order == 2 ? 2.0 : (order == 4 ? 12.0 : 60.0);
  p.fx_sig[0] = -hix / den;
  p.fx_sig[1] = -hiy / den;
  p.fx_isig[0] = -den / hix;
  p.fx_isig[1] = -den / hiy;
  p.fx_rho = hiy / hix;
  p.fx_square = hix == hiy ? 1 : 0;
  p.fx_sigp = p.fx_sig[0];
  const double sg[3] = {p.fx_sig[0], p.fx_sig[1], p.fx_sigp};
  for (int c = 0; c < 3; c++) {
    p.fx_ca[c] = p.c_acc * sg[c];
    p.fx_cw[c] = p.c_w * sg[c];
  }
}

// Streaming multiprocessors of the current device (cached per device).
int device_sm_count();

template <typename T>
cudaError_t launch_wave_o2(int kind, int stage, const WaveMaps& m, const WaveParams<T>& prm, dim3 grid, cudaStream_t s);
template <typename T>
cudaError_t launch_wave_o4(int kind, int stage, const WaveMaps& m, const WaveParams<T>& prm, dim3 grid, cudaStream_t s);
template <typename T>
cudaError_t launch_wave_o6(int kind, int stage, const WaveMaps& m, const WaveParams<T>& prm, dim3 grid, cudaStream_t s);

// Sets the dynamic shared-memory opt-in of every stage kernel of (order, kind).
template <typename T> cudaError_t configure_wave_o2(int kind);
template <typename T> cudaError_t configure_wave_o4(int kind);
template <typename T> cudaError_t configure_wave_o6(int kind);
template <typename T> inline cudaError_t configure_wave(int order, int kind) {
  return order == 2 ? configure_wave_o2<T>(kind) : (order == 4 ? configure_wave_o4<T>(kind) : configure_wave_o6<T>(kind));
}

template <typename T>
inline cudaError_t launch_wave(int order, int kind, int stage, const WaveMaps& m, const WaveParams<T>& prm,
                               cudaStream_t s) {
  // persistent grid: one CTA per SM, each walking the tiles with a fixed stride
  const int ty = wave_tile_height((int)sizeof(T), kind);
  const long long ntiles = (long long)((prm.nx + kWaveTX - 1) / kWaveTX) * ((prm.ny + ty - 1) / ty);
  const int nsm = device_sm_count();
  const dim3 grid((unsigned)(ntiles < nsm ? ntiles : nsm));
  switch (order) {
    case 2: return launch_wave_o2<T>(kind, stage, m, prm, grid, s);
    case 4: return launch_wave_o4<T>(kind, stage, m, prm, grid, s);
    case 6: return launch_wave_o6<T>(kind, stage, m, prm, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

// Shared memory bytes of one wave tile (for occupancy reports).
int wave_smem_bytes(int order, bool fp32);

template <typename T>
cudaError_t launch_line(int order, int kind, int stage, const LineParams<T>& prm, cudaStream_t s);

// The 3D wave stage kernel (wave3d.cu).
template <typename T>
cudaError_t launch_wave3d(int order, int stage, const Wave3Params<T>& prm, cudaStream_t s);
// Shared-memory opt-in of the 3D stage kernels of one order (outside stream capture).
template <typename T> cudaError_t configure_wave3d(int order);

// Batched stage kernels (wave_batch_inst.cu, one unit per order): configuration
// `cfg` of the wave (wave = true) or advection table of wave_batch.cuh.
#define SBP_DECLARE_BATCH(o)                                                                                    \
  template <typename T> cudaError_t configure_batch_o##o(bool wave, int cfg);                                   \
  template <typename T>                                                                                         \
  cudaError_t launch_batch_o##o(bool wave, int stage, int cfg, const void* insts, const CUtensorMap* maps,      \
                                const BatchTile* tiles, int ntiles, int rk, int* err, unsigned grid, cudaStream_t s);
SBP_DECLARE_BATCH(2)
SBP_DECLARE_BATCH(4)
SBP_DECLARE_BATCH(6)
#undef SBP_DECLARE_BATCH

// The configuration `cfg` of a group's table (wave or advection kernel).
template <typename T> inline BatchCfg batch_cfg(bool wave, int cfg) {
  return wave ? BatchCfgTable<T>::wave[cfg] : BatchCfgTable<T>::adv[cfg];
}

template <typename T> inline cudaError_t configure_batch(int order, bool wave, int cfg) {
  if (cfg < 0 || cfg >= kBatchCfgs) return cudaErrorInvalidValue;
  return order == 2 ? configure_batch_o2<T>(wave, cfg)
                    : (order == 4 ? configure_batch_o4<T>(wave, cfg) : configure_batch_o6<T>(wave, cfg));
}
// One stage of one group: a persistent grid of (CTAs per SM) x SMs, or one CTA per
// tile when the group has fewer tiles.
template <typename T>
inline cudaError_t launch_batch(int order, bool wave, int stage, int cfg, const void* insts, const CUtensorMap* maps,
                                const BatchTile* tiles, int ntiles, int rk, int* err, cudaStream_t s) {
  if (cfg < 0 || cfg >= kBatchCfgs) return cudaErrorInvalidValue;
  const int slots = device_sm_count() * batch_cfg<T>(wave, cfg).ctas;
  const unsigned grid = (unsigned)(ntiles < slots ? ntiles : slots);
  switch (order) {
    case 2: return launch_batch_o2<T>(wave, stage, cfg, insts, maps, tiles, ntiles, rk, err, grid, s);
    case 4: return launch_batch_o4<T>(wave, stage, cfg, insts, maps, tiles, ntiles, rk, err, grid, s);
    case 6: return launch_batch_o6<T>(wave, stage, cfg, insts, maps, tiles, ntiles, rk, err, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

// AoS FP64 (reference layout) <-> SoA planes of T with a row pitch.
template <typename T>
cudaError_t launch_pack(const double* aos, T* soa, int nx, int ny, int dofs, long long pitch, long long plane,
                        cudaStream_t s);
template <typename T>
cudaError_t launch_unpack(const T* soa, double* aos, int nx, int ny, int dofs, long long pitch, long long plane,
                          cudaStream_t s);

// Number of partial sums the reductions write (scratch of 2*kReduceBlocks doubles).
constexpr int kReduceBlocks = 592;  // 4 blocks per SM on 148-152 SMs

// Sum of squared differences and max |difference| between the SoA state and
// an AoS FP64 array: out[0] = sum e^2, out[1] = max |e|.
template <typename T>
cudaError_t launch_error_norms(const T* soa, const double* aos, int nx, int ny, int dofs, long long pitch,
                               long long plane, double* partial, double* out, cudaStream_t s);
// Energy norm squared sum_c sum_j sum_i hy*wy_j * hx*wx_i * v^2 with the
// closure quadrature at both ends of each direction (of each block when
// ysplit > 0): out[0].
// 3D (nz > 1): ny*nz rows, the z quadrature weight hz * w_k of slab k = row / ny as a third factor.
template <typename T>
cudaError_t launch_hnorm(const T* soa, int nx, int ny, int dofs, long long pitch, long long plane, int order,
                         double hx, double hy, int ysplit, double* partial, double* out, cudaStream_t s,
                         int nz = 1, double hz = 1.0);

// ---------------------------------------------------------------- RK45 (rk45.cu)
// Buffers of the adaptive Runge-Kutta-Fehlberg 4(5) integrator (FP64 SoA planes
// of the context's layout).
struct Rk45Buffers {
  int nx, ny, dofs;
  long long pitch, plane;
  double* u;        // current solution
  double* w;        // stage input
  double* k[6];     // stage derivatives
  double* unew;     // candidate solution of the attempt
  double* partial;  // kReduceBlocks partial sums of the weighted error
};

enum Rk45Status : int { RK45_OK = 0, RK45_STEP_LIMIT = 1, RK45_NONFINITE = 2, RK45_REJECTED = 3 };

// Controller state in device memory; the stage kernels read t and h (adjacent,
// in this order) for time-dependent forcing, and `done` to skip their work.
struct Rk45Ctrl {
  double t, h;  // time reached, step of the next attempt
  double t_end, atol, rtol, safety, reject_safety, clip_lo, clip_hi, dt_min, dt_max;
  double wlte;  // weighted error of the last attempt
  double n;     // scalars in the error norm
  long long accepted, rejected, max_steps;
  int max_reject, rejects_in_row;
  int done;          // stop: every kernel of later attempts returns at entry
  int copy_pending;  // the last attempt was accepted: its solution replaces u
  int last_accepted, final_step, status;
};

// w = u + h sum_{j<=stage} a[stage][j] k_j (the input of stage `stage` + 1).
cudaError_t launch_rk45_combine(int stage, const Rk45Buffers& b, const Rk45Ctrl* ctrl, cudaStream_t s);
// Candidate solution and error partial sums, the controller, and the accept copy.
cudaError_t launch_rk45_finish(const Rk45Buffers& b, Rk45Ctrl* ctrl, cudaStream_t s);
// The controller over `nparts` partial sums already in b.partial, and the accept copy
// (after the fused wave stage ST_RKF6 wrote the candidate and one partial per CTA).
cudaError_t launch_rk45_control(const Rk45Buffers& b, int nparts, Rk45Ctrl* ctrl, cudaStream_t s);

// FP64 fused-multiply-add throughput probe: each thread runs `iters`
// iterations of 8 independent DFMA chains; result written to out[0].
cudaError_t launch_dfma_probe(double* out, int blocks, int threads, int iters, cudaStream_t s);

}  // namespace sbp
