// sbp_device.cuh -- device-side building blocks shared by the SBP kernels:
// operator shapes per order, TMA / mbarrier wrappers (inline PTX, sm_103a) with
// bounded waits, and the launch-parameter structs.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace sbp {

// Shapes of the central SBP first-derivative operators
// (code/include/sbpops/D1_central.h:243-273): interior stencil width, number
// of closure rows, closure row width.
template <int ORD> struct OpShape;
template <> struct OpShape<2> { static constexpr int W = 3, CS = 1, CW = 2; };
template <> struct OpShape<4> { static constexpr int W = 5, CS = 4, CW = 6; };
template <> struct OpShape<6> { static constexpr int W = 7, CS = 6, CW = 9; };

// Scaled operator taps for one direction, filled on the host: taps[s] is
// scale * interior_stencil[s] and cls[r][s] is scale * closure_stencils[r][s],
// where scale is -hi (the sign of every wave/advection RHS term folded in).
template <typename T> struct DirTaps {
  T taps[7];
  T cls[6][9];
};

// Error bits a kernel can raise (read back by the host after the launch).
enum : int {
  ERR_TMA_TIMEOUT = 1,     // an mbarrier wait for a TMA tile gave up
  ERR_BAD_LAUNCH = 2,      // grid/tile arithmetic inconsistent with the params
};

// Upper bound for one mbarrier wait, in nanoseconds of %globaltimer. A tile
// load takes microseconds; 200 ms means the copy will not complete.
constexpr uint64_t kWaitLimitNs = 200ull * 1000ull * 1000ull;

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// A plain arrive (count 1) on an mbarrier.
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of the barrier with a time limit (nanoseconds of
// %globaltimer; 0 means kWaitLimitNs). Returns false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns = 0) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t lim = limit_ns ? limit_ns : kWaitLimitNs;
  const uint64_t t0 = globaltimer_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (globaltimer_ns() - t0 > lim) return false;
  }
}

// 3D tiled TMA load (x innermost) into shared memory, completion counted in
// bytes on `bar`. x * sizeof(element) must be a multiple of 16: every caller
// passes x = tile origin minus a halo that is a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_3d(void* smem_dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(smem_dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

// Untiled bulk copy global -> shared (cp.async.bulk), completion counted in bytes
// on `bar`. Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void* smem_dst, const void* gsrc, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(smem_dst)),
               "l"(reinterpret_cast<uint64_t>(gsrc)), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Streaming loads/stores for values touched once per stage.
template <typename T> __device__ __forceinline__ T ld_stream(const T* p) { return __ldcs(p); }
template <typename T> __device__ __forceinline__ void st_stream(T* p, T v) { __stcs(p, v); }

}  // namespace sbp
