// wave_batch_inst.cu -- instantiations and launchers of the batched stage
// kernels for one SBP order (compiled once per order with -DSBP_ORDER=2/4/6).
// Tile heights offered to the autotuner: FP64 8 or 16 rows, FP32 16 or 32.
#include "launch.h"

#ifndef SBP_ORDER
#error "compile with -DSBP_ORDER=2, 4 or 6"
#endif

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)

namespace sbp {

namespace {

template <typename T, int STAGE, int TY>
constexpr int batch_smem() {
  return BatchWaveTile<T, SBP_ORDER, STAGE, TY>::SMEM;
}

template <typename T, int TY>
cudaError_t configure_ty() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(wave_batch_stage_kernel<T, SBP_ORDER, ST_FIRST, TY>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, batch_smem<T, ST_FIRST, TY>())) !=
      cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(wave_batch_stage_kernel<T, SBP_ORDER, ST_MID, TY>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, batch_smem<T, ST_MID, TY>())) !=
      cudaSuccess)
    return e;
  return cudaFuncSetAttribute(wave_batch_stage_kernel<T, SBP_ORDER, ST_LAST, TY>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, batch_smem<T, ST_LAST, TY>());
}

template <typename T, int TY>
cudaError_t launch_ty(int stage, const BatchWave<T>* insts, const CUtensorMap* maps, const BatchTile* tiles, int ntiles,
                      int rk, int* err, unsigned grid, cudaStream_t s) {
  switch (stage) {
    case ST_FIRST:
      wave_batch_stage_kernel<T, SBP_ORDER, ST_FIRST, TY>
          <<<grid, BatchWaveTile<T, SBP_ORDER, ST_FIRST, TY>::THREADS, batch_smem<T, ST_FIRST, TY>(), s>>>(insts, maps, tiles, ntiles, rk, err);
      break;
    case ST_MID:
      wave_batch_stage_kernel<T, SBP_ORDER, ST_MID, TY>
          <<<grid, BatchWaveTile<T, SBP_ORDER, ST_MID, TY>::THREADS, batch_smem<T, ST_MID, TY>(), s>>>(insts, maps, tiles, ntiles, rk, err);
      break;
    case ST_LAST:
      wave_batch_stage_kernel<T, SBP_ORDER, ST_LAST, TY>
          <<<grid, BatchWaveTile<T, SBP_ORDER, ST_LAST, TY>::THREADS, batch_smem<T, ST_LAST, TY>(), s>>>(insts, maps, tiles, ntiles, rk, err);
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

template <>
cudaError_t CAT(configure_wave_batch_o, SBP_ORDER)<double>(int ty) {
  return ty == 8 ? configure_ty<double, 8>() : (ty == 16 ? configure_ty<double, 16>() : cudaErrorInvalidValue);
}
template <>
cudaError_t CAT(configure_wave_batch_o, SBP_ORDER)<float>(int ty) {
  return ty == 16 ? configure_ty<float, 16>() : (ty == 32 ? configure_ty<float, 32>() : cudaErrorInvalidValue);
}

template <>
cudaError_t CAT(launch_wave_batch_o, SBP_ORDER)<double>(int stage, int ty, const BatchWave<double>* insts,
                                                        const CUtensorMap* maps, const BatchTile* tiles, int ntiles, int rk,
                                                        int* err, unsigned grid, cudaStream_t s) {
  if (ty == 8) return launch_ty<double, 8>(stage, insts, maps, tiles, ntiles, rk, err, grid, s);
  if (ty == 16) return launch_ty<double, 16>(stage, insts, maps, tiles, ntiles, rk, err, grid, s);
  return cudaErrorInvalidValue;
}
template <>
cudaError_t CAT(launch_wave_batch_o, SBP_ORDER)<float>(int stage, int ty, const BatchWave<float>* insts,
                                                       const CUtensorMap* maps, const BatchTile* tiles, int ntiles, int rk,
                                                       int* err, unsigned grid, cudaStream_t s) {
  if (ty == 16) return launch_ty<float, 16>(stage, insts, maps, tiles, ntiles, rk, err, grid, s);
  if (ty == 32) return launch_ty<float, 32>(stage, insts, maps, tiles, ntiles, rk, err, grid, s);
  return cudaErrorInvalidValue;
}

template <typename T>
static cudaError_t adv_launch(int stage, const BatchLine<T>* insts, const BatchTile* tiles, int ntiles, int rk,
                              cudaStream_t s) {
  const dim3 block(kLineTileX, kLineThreadsY);
  switch (stage) {
    case ST_FIRST: adv_batch_stage_kernel<T, SBP_ORDER, ST_FIRST><<<ntiles, block, 0, s>>>(insts, tiles, rk); break;
    case ST_MID: adv_batch_stage_kernel<T, SBP_ORDER, ST_MID><<<ntiles, block, 0, s>>>(insts, tiles, rk); break;
    case ST_LAST: adv_batch_stage_kernel<T, SBP_ORDER, ST_LAST><<<ntiles, block, 0, s>>>(insts, tiles, rk); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <>
cudaError_t CAT(launch_adv_batch_o, SBP_ORDER)<double>(int stage, const BatchLine<double>* insts, const BatchTile* tiles,
                                                       int ntiles, int rk, cudaStream_t s) {
  return adv_launch<double>(stage, insts, tiles, ntiles, rk, s);
}
template <>
cudaError_t CAT(launch_adv_batch_o, SBP_ORDER)<float>(int stage, const BatchLine<float>* insts, const BatchTile* tiles,
                                                      int ntiles, int rk, cudaStream_t s) {
  return adv_launch<float>(stage, insts, tiles, ntiles, rk, s);
}

}  // namespace sbp
