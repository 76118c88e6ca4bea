// wave_batch_inst.cu -- instantiations and launchers of the batched stage
// kernels for one SBP order (compiled once per order with -DSBP_ORDER=2/4/6):
// every configuration of the wave and advection tables (wave_batch.cuh) for
// the three RK4 stage kinds, FP32 and FP64.
#include "launch.h"

#ifndef SBP_ORDER
#error "compile with -DSBP_ORDER=2, 4 or 6"
#endif

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)

namespace sbp {

namespace {

template <typename T, int STAGE, int CFG>
cudaError_t configure_wave_one() {
  if constexpr (batch_wave_cfg<T, CFG>().conv > 0) {
    static_assert(sizeof(T) == 8, "the fixed-point stencils are an FP64 form");
    return cudaFuncSetAttribute(wave_batch_fixed_kernel<SBP_ORDER, STAGE, CFG>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                BatchWaveTile<T, SBP_ORDER, STAGE, CFG>::SMEM);
  } else {
    return cudaFuncSetAttribute(wave_batch_stage_kernel<T, SBP_ORDER, STAGE, CFG>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                BatchWaveTile<T, SBP_ORDER, STAGE, CFG>::SMEM);
  }
}

template <typename T, int STAGE, int CFG>
cudaError_t configure_adv_one() {
  return cudaFuncSetAttribute(adv_batch_stage_kernel<T, SBP_ORDER, STAGE, CFG>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, AdvTile<T, SBP_ORDER, STAGE, CFG>::SMEM);
}

template <typename T, int CFG>
cudaError_t configure_cfg(bool wave) {
  cudaError_t e;
  if (wave) {
    if ((e = configure_wave_one<T, ST_FIRST, CFG>()) != cudaSuccess) return e;
    if ((e = configure_wave_one<T, ST_MID, CFG>()) != cudaSuccess) return e;
    return configure_wave_one<T, ST_LAST, CFG>();
  }
  if ((e = configure_adv_one<T, ST_FIRST, CFG>()) != cudaSuccess) return e;
  if ((e = configure_adv_one<T, ST_MID, CFG>()) != cudaSuccess) return e;
  return configure_adv_one<T, ST_LAST, CFG>();
}

template <typename T, int STAGE, int CFG>
void launch_wave_one(const BatchWave<T>* insts, const CUtensorMap* maps, const BatchTile* tiles, int ntiles, int rk,
                     int* err, unsigned grid, cudaStream_t s) {
  using Tile = BatchWaveTile<T, SBP_ORDER, STAGE, CFG>;
  if constexpr (batch_wave_cfg<T, CFG>().conv > 0)
    wave_batch_fixed_kernel<SBP_ORDER, STAGE, CFG><<<grid, Tile::THREADS, Tile::SMEM, s>>>(insts, maps, tiles, ntiles,
                                                                                         rk, err);
  else
    wave_batch_stage_kernel<T, SBP_ORDER, STAGE, CFG><<<grid, Tile::THREADS, Tile::SMEM, s>>>(insts, maps, tiles,
                                                                                              ntiles, rk, err);
}

template <typename T, int STAGE, int CFG>
void launch_adv_one(const BatchLine<T>* insts, const CUtensorMap* maps, const BatchTile* tiles, int ntiles, int rk,
                    int* err, unsigned grid, cudaStream_t s) {
  using Tile = AdvTile<T, SBP_ORDER, STAGE, CFG>;
  adv_batch_stage_kernel<T, SBP_ORDER, STAGE, CFG><<<grid, Tile::THREADS, Tile::SMEM, s>>>(insts, maps, tiles, ntiles,
                                                                                           rk, err);
}

template <typename T, int CFG>
cudaError_t launch_cfg(bool wave, int stage, const void* insts, const CUtensorMap* maps, const BatchTile* tiles,
                       int ntiles, int rk, int* err, unsigned grid, cudaStream_t s) {
  if (wave) {
    const BatchWave<T>* w = static_cast<const BatchWave<T>*>(insts);
    switch (stage) {
      case ST_FIRST: launch_wave_one<T, ST_FIRST, CFG>(w, maps, tiles, ntiles, rk, err, grid, s); break;
      case ST_MID: launch_wave_one<T, ST_MID, CFG>(w, maps, tiles, ntiles, rk, err, grid, s); break;
      case ST_LAST: launch_wave_one<T, ST_LAST, CFG>(w, maps, tiles, ntiles, rk, err, grid, s); break;
      default: return cudaErrorInvalidValue;
    }
  } else {
    const BatchLine<T>* l = static_cast<const BatchLine<T>*>(insts);
    switch (stage) {
      case ST_FIRST: launch_adv_one<T, ST_FIRST, CFG>(l, maps, tiles, ntiles, rk, err, grid, s); break;
      case ST_MID: launch_adv_one<T, ST_MID, CFG>(l, maps, tiles, ntiles, rk, err, grid, s); break;
      case ST_LAST: launch_adv_one<T, ST_LAST, CFG>(l, maps, tiles, ntiles, rk, err, grid, s); break;
      default: return cudaErrorInvalidValue;
    }
  }
  return cudaGetLastError();
}

}  // namespace

static_assert(kBatchCfgs == 4, "the switches below cover four configurations");

template <typename T>
cudaError_t CAT(configure_batch_o, SBP_ORDER)(bool wave, int cfg) {
  switch (cfg) {
    case 0: return configure_cfg<T, 0>(wave);
    case 1: return configure_cfg<T, 1>(wave);
    case 2: return configure_cfg<T, 2>(wave);
    case 3: return configure_cfg<T, 3>(wave);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
cudaError_t CAT(launch_batch_o, SBP_ORDER)(bool wave, int stage, int cfg, const void* insts, const CUtensorMap* maps,
                                          const BatchTile* tiles, int ntiles, int rk, int* err, unsigned grid,
                                          cudaStream_t s) {
  switch (cfg) {
    case 0: return launch_cfg<T, 0>(wave, stage, insts, maps, tiles, ntiles, rk, err, grid, s);
    case 1: return launch_cfg<T, 1>(wave, stage, insts, maps, tiles, ntiles, rk, err, grid, s);
    case 2: return launch_cfg<T, 2>(wave, stage, insts, maps, tiles, ntiles, rk, err, grid, s);
    case 3: return launch_cfg<T, 3>(wave, stage, insts, maps, tiles, ntiles, rk, err, grid, s);
    default: return cudaErrorInvalidValue;
  }
}

template cudaError_t CAT(configure_batch_o, SBP_ORDER)<float>(bool, int);
template cudaError_t CAT(configure_batch_o, SBP_ORDER)<double>(bool, int);
template cudaError_t CAT(launch_batch_o, SBP_ORDER)<float>(bool, int, int, const void*, const CUtensorMap*,
                                                          const BatchTile*, int, int, int*, unsigned, cudaStream_t);
template cudaError_t CAT(launch_batch_o, SBP_ORDER)<double>(bool, int, int, const void*, const CUtensorMap*,
                                                           const BatchTile*, int, int, int*, unsigned, cudaStream_t);

}  // namespace sbp
