// wave2d_inst.cu -- instantiations and launcher of the fused wave stage kernel
// for one SBP order. The build compiles this file once per order with
// -DSBP_ORDER=2, 4 or 6 so the three orders compile in parallel.
#include "launch.h"

#ifndef SBP_ORDER
#error "compile with -DSBP_ORDER=2, 4 or 6"
#endif

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define LAUNCH_WAVE CAT(launch_wave_o, SBP_ORDER)
#define CONFIGURE_WAVE CAT(configure_wave_o, SBP_ORDER)

namespace sbp {

namespace {

// The fixed-point FP64 stages with converter warps run their own kernel
// (wave_fixed_kernel); every other stage runs wave_stage_kernel.
template <typename T, int KIND, int STAGE>
constexpr bool uses_fixed_kernel() {
  return WaveStageTile<T, SBP_ORDER, KIND, STAGE>::FIX && WaveStageTile<T, SBP_ORDER, KIND, STAGE>::CONV > 0;
}

template <typename T, int KIND, int STAGE>
cudaError_t configure_one() {
  if constexpr (uses_fixed_kernel<T, KIND, STAGE>())
    return cudaFuncSetAttribute(wave_fixed_kernel<SBP_ORDER, STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                WaveStageTile<T, SBP_ORDER, KIND, STAGE>::SMEM);
  else
    return cudaFuncSetAttribute(wave_stage_kernel<T, SBP_ORDER, KIND, STAGE>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                WaveStageTile<T, SBP_ORDER, KIND, STAGE>::SMEM);
}

template <typename T, int KIND>
cudaError_t configure_kind() {
  cudaError_t e;
  if ((e = configure_one<T, KIND, ST_RHS>()) != cudaSuccess) return e;
  if ((e = configure_one<T, KIND, ST_FIRST>()) != cudaSuccess) return e;
  if ((e = configure_one<T, KIND, ST_MID>()) != cudaSuccess) return e;
  if ((e = configure_one<T, KIND, ST_LAST>()) != cudaSuccess) return e;
  if constexpr (sizeof(T) == 8) {  // the Fehlberg stages (FP64 only)
    if ((e = configure_one<T, KIND, ST_RKF1>()) != cudaSuccess) return e;
    if ((e = configure_one<T, KIND, ST_RKF1 + 1>()) != cudaSuccess) return e;
    if ((e = configure_one<T, KIND, ST_RKF1 + 2>()) != cudaSuccess) return e;
    if ((e = configure_one<T, KIND, ST_RKF1 + 3>()) != cudaSuccess) return e;
    if ((e = configure_one<T, KIND, ST_RKF1 + 4>()) != cudaSuccess) return e;
    if ((e = configure_one<T, KIND, ST_RKF6>()) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename T, int KIND, int STAGE>
cudaError_t launch_one(const WaveMaps& m, const WaveParams<T>& prm, dim3 grid, cudaStream_t s) {
  using Tile = WaveStageTile<T, SBP_ORDER, KIND, STAGE>;
  if constexpr (uses_fixed_kernel<T, KIND, STAGE>())
    wave_fixed_kernel<SBP_ORDER, STAGE><<<grid, Tile::THREADS, Tile::SMEM, s>>>(m.p, m.u, m.v, m.n, m.a, m.c, m.k, prm);
  else
    wave_stage_kernel<T, SBP_ORDER, KIND, STAGE>
        <<<grid, Tile::THREADS, Tile::SMEM, s>>>(m.p, m.u, m.v, m.n, m.a, m.c, m.k, prm);
  return cudaGetLastError();
}

template <typename T, int KIND>
cudaError_t launch_kind(int stage, const WaveMaps& m, const WaveParams<T>& prm, dim3 grid, cudaStream_t s) {
  switch (stage) {
    case ST_RHS: return launch_one<T, KIND, ST_RHS>(m, prm, grid, s);
    case ST_FIRST: return launch_one<T, KIND, ST_FIRST>(m, prm, grid, s);
    case ST_MID: return launch_one<T, KIND, ST_MID>(m, prm, grid, s);
    case ST_LAST: return launch_one<T, KIND, ST_LAST>(m, prm, grid, s);
    default: break;
  }
  if constexpr (sizeof(T) == 8) {
    switch (stage) {
      case ST_RKF1: return launch_one<T, KIND, ST_RKF1>(m, prm, grid, s);
      case ST_RKF1 + 1: return launch_one<T, KIND, ST_RKF1 + 1>(m, prm, grid, s);
      case ST_RKF1 + 2: return launch_one<T, KIND, ST_RKF1 + 2>(m, prm, grid, s);
      case ST_RKF1 + 3: return launch_one<T, KIND, ST_RKF1 + 3>(m, prm, grid, s);
      case ST_RKF1 + 4: return launch_one<T, KIND, ST_RKF1 + 4>(m, prm, grid, s);
      case ST_RKF6: return launch_one<T, KIND, ST_RKF6>(m, prm, grid, s);
      default: break;
    }
  }
  return cudaErrorInvalidValue;
}

}  // namespace

template <>
cudaError_t CONFIGURE_WAVE<double>(int kind) {
  switch (kind) {
    case WK_HOM: return configure_kind<double, WK_HOM>();
    case WK_VAR: return configure_kind<double, WK_VAR>();
    case WK_MMS: return configure_kind<double, WK_MMS>();
    default: return cudaErrorInvalidValue;
  }
}

template <>
cudaError_t CONFIGURE_WAVE<float>(int kind) {
  switch (kind) {
    case WK_HOM: return configure_kind<float, WK_HOM>();
    case WK_VAR: return configure_kind<float, WK_VAR>();
    default: return cudaErrorInvalidValue;
  }
}

template <>
cudaError_t LAUNCH_WAVE<double>(int kind, int stage, const WaveMaps& m, const WaveParams<double>& prm, dim3 grid,
                                cudaStream_t s) {
  switch (kind) {
    case WK_HOM: return launch_kind<double, WK_HOM>(stage, m, prm, grid, s);
    case WK_VAR: return launch_kind<double, WK_VAR>(stage, m, prm, grid, s);
    case WK_MMS: return launch_kind<double, WK_MMS>(stage, m, prm, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

template <>
cudaError_t LAUNCH_WAVE<float>(int kind, int stage, const WaveMaps& m, const WaveParams<float>& prm, dim3 grid,
                               cudaStream_t s) {
  switch (kind) {
    case WK_HOM: return launch_kind<float, WK_HOM>(stage, m, prm, grid, s);
    case WK_VAR: return launch_kind<float, WK_VAR>(stage, m, prm, grid, s);
    default: return cudaErrorInvalidValue;  // the manufactured-solution problem is FP64 only
  }
}

}  // namespace sbp
