// cnn.cu -- the learned correction: a 4-layer 3x3 convolutional network
// (24 -> 32 -> 32 -> 32 -> 3 channels, ReLU between layers) trained and run on
// the GPU by the kernels in this file. No counterpart in the reference.
//
// Tensors are NHWC. Activations and weights are BF16; every product is
// accumulated in FP32 on the tensor cores; master weights, biases and Adam
// moments are FP32. Channel counts are padded to multiples of 16 (the MMA K
// step): input 24 -> 32, output 3 -> 16; the padding carries zeros.
//
//   conv3x3_tc_kernel     implicit GEMM on tcgen05 (TMA tiles, tensor-memory
//                         accumulator), M = 128 pixels, N = output channels,
//                         K = 9 taps x input channels; also computes the input
//                         gradient (dgrad) with the spatially flipped,
//                         transposed weights.
//   conv3x3_wgrad_tc_kernel  weight gradient on tcgen05, K = pixels: four taps'
//                         shifted input tiles stacked along M (MN-major operands),
//                         accumulated over all of a CTA's pixel tiles in tensor
//                         memory; wgrad_reduce_kernel adds the CTAs' sums to dw in
//                         CTA order (repeatable bits).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "../../include/sbpgpu.h"
#include "sbp_device.cuh"

namespace sbp {
namespace cnn {

typedef __nv_bfloat16 bf16;

constexpr int kLayers = 4;
constexpr int kCin[kLayers] = {32, 32, 32, 32};   // padded input channels
constexpr int kCout[kLayers] = {32, 32, 32, 16};  // padded output channels
constexpr int kInReal = 24, kOutReal = 3;

__device__ __forceinline__ uint32_t pack_pair(bf16 lo, bf16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}


// ---------------------------------------------------------------- tcgen05 convolution
// The forward and input-gradient 3x3 convolutions on the 5th-generation tensor cores:
// an implicit GEMM per 128-pixel tile (th x tw pixels of one image), M = 128 pixels,
// N = COUT, K = 9 taps x CIN. TMA loads each tap's shifted input tile (a 4D box
// {CIN, tw, th, 1} of the NHWC activations: the image border comes back as zeros)
// and each tap's weight tile into shared memory, rows of CIN BF16 values swizzled
// by the TMA (64-byte swizzle for 32 channels, 32-byte for 16) -- the K-major
// layout the MMA's shared-memory descriptors describe. One thread issues
// tcgen05.mma (kind::f16, BF16 inputs, FP32 accumulator in tensor memory) tap by
// tap as the tiles land, K = 16 per instruction; tcgen05.commit signals the
// epilogue, where each warp reads its 32 accumulator lanes (pixels) with
// tcgen05.ld, adds the bias, applies ReLU and stores. Every wait is bounded.

// Shared-memory descriptor of a K-major operand tile with rows of `rowb` bytes
// swizzled in 8-row atoms (stride between atoms: 8 rows), tcgen05 version.
__device__ __forceinline__ uint64_t umma_smem_desc(uint32_t saddr, uint32_t atom_bytes, uint32_t layout) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);  // start address
  d |= (uint64_t)1u << 16;                           // leading offset: unused by swizzled K-major tiles
  d |= (uint64_t)((atom_bytes >> 4) & 0x3FFFu) << 32;  // stride offset: one 8-row atom
  d |= (uint64_t)1u << 46;                           // descriptor version of tcgen05
  d |= (uint64_t)layout << 61;                       // swizzle mode
  return d;
}

// The same for an MN-major operand: rows along K of one swizzle span of M (or N)
// values; `lead` = byte stride between swizzle spans along M, `stride` = between
// 8-row groups along K.
__device__ __forceinline__ uint64_t umma_smem_desc_mn(uint32_t saddr, uint32_t lead, uint32_t stride,
                                                      uint32_t layout) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lead >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((stride >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1u << 46;
  d |= (uint64_t)layout << 61;
  return d;
}

// Instruction descriptor of kind::f16: BF16 A and B (both K-major), FP32 D, M x N.
constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t"
      "}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive accumulator columns of this thread's lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
      : "memory");
}

// Shared-memory layout of conv3x3_tc_kernel: a ring of NS tap tiles (128 pixel rows
// of CIN BF16), the nine taps' weight tiles (COUT rows of CIN), barriers and the
// tensor-memory address; tiles 1024-byte aligned (whole swizzle atoms).
template <int CIN, int COUT>
struct TcConv {
  static_assert(CIN == 16 || CIN == 32, "input channels: one or two K steps of 16 per tap");
  static_assert(COUT == 16 || COUT == 32, "output channels: the MMA's N");
  static constexpr int ROWB = CIN * 2;  // bytes per row: the swizzle span
  static constexpr uint32_t LAYOUT = CIN == 32 ? 4u : 6u;  // 64-byte / 32-byte swizzle
  static constexpr uint32_t ATOM = 8 * ROWB;
  static constexpr int NS = 9;  // tap tiles in flight: one pixel tile per CTA, two CTAs per SM
  static constexpr int CTAS = 2;  // resident CTAs per SM (measured at 8 x 258 x 257, forward pass:
                                  // 0.198 ms; one CTA with 18 slots 0.310 ms, one tile per CTA
                                  // 0.271 ms, the mma.sync form 0.471 ms)
  static constexpr int A_BYTES = 128 * ROWB, B_BYTES = COUT * ROWB;
  static constexpr int OFF_B = NS * A_BYTES;
  static constexpr int OFF_BAR = OFF_B + ((9 * B_BYTES + 1023) / 1024) * 1024;
  // full[NS], empty[NS], wbar, accfull[2], accempty[2], done; then the tensor-memory address
  static constexpr int NBAR = 2 * NS + 6;
  static constexpr int SMEM = OFF_BAR + 8 * NBAR + 16 + 1024;  // + alignment slack of the dynamic base
  static constexpr uint32_t IDESC = umma_idesc_bf16(128, COUT);
  static constexpr int THREADS = 192;  // producer, MMA issuer, four epilogue warps
  static_assert(A_BYTES % 1024 == 0 && B_BYTES % 256 == 0, "tiles start on swizzle atoms");
  static_assert(CTAS * (SMEM + 1024) <= 228 * 1024, "shared memory");
};

// y[p][n] = act(bias[n] + sum_{tap,c} x[p + off(tap)][c] * w[n][tap][c]); x through xmap
// ({CIN, W, H, B}), w through wmap ({CIN, 9, COUT}). Persistent, two CTAs per SM: a CTA
// takes every gridDim.x-th 128-pixel tile (th rows of tw pixels). Warp roles: warp 0 loads the weights
// once, then each tile's nine shifted tap tiles into a ring of NS slots; warp 1 (which owns
// the tensor memory) issues each tap's MMAs as its tile lands, frees the slot with
// tcgen05.commit, and commits each pixel tile into one of two accumulators (32 columns
// each); warps 2-5 read an accumulator (warp w: lanes 32 (w % 4) ..), release it, and add
// bias, apply ReLU and store while the next tile accumulates in the other. Bounded waits.
template <int CIN, int COUT, bool RELU, bool OUT_F32>
__global__ void __launch_bounds__(TcConv<CIN, COUT>::THREADS, TcConv<CIN, COUT>::CTAS)
    conv3x3_tc_kernel(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap wmap,
                      const float* __restrict__ bias, void* __restrict__ y, int B, int H, int W, int tw, int th,
                      int* err) {
  using L = TcConv<CIN, COUT>;
  constexpr int NS = L::NS;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((1024 - (smem_addr(smem_raw) & 1023)) & 1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L::OFF_BAR);
  uint64_t* empty = full + NS;
  uint64_t* wbar = empty + NS;
  uint64_t* accfull = wbar + 1;
  uint64_t* accempty = accfull + 2;
  uint64_t* done = accempty + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntw = (W + tw - 1) / tw, nth = (H + th - 1) / th;
  const int ntiles = B * nth * ntw;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(wbar, 1);
    for (int s = 0; s < 2; s++) {
      mbar_init(&accfull[s], 1);
      mbar_init(&accempty[s], 4);
    }
    mbar_init(done, 1);
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tslot, 64);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0) {  // ---- loads
    if (lane == 0) {
      mbar_arrive_expect_tx(wbar, 9 * L::B_BYTES);
      for (int t = 0; t < 9; t++) tma_load_3d(smem + L::OFF_B + t * L::B_BYTES, &wmap, 0, t, 0, wbar);
      int k = 0;
      bool ok = true;
      for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
        const int w0 = (tile % ntw) * tw, h0 = ((tile / ntw) % nth) * th, b = tile / (ntw * nth);
        for (int t = 0; t < 9; t++, k++) {
          const int s = k % NS;
          if (k >= NS && !mbar_wait_bounded(&empty[s], ((k / NS) - 1) & 1)) {
            atomicOr(err, 1);
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(&full[s], L::A_BYTES);
          tma_load_4d(smem + s * L::A_BYTES, &xmap, 0, w0 + t % 3 - 1, h0 + t / 3 - 1, b, &full[s]);
        }
      }
      // no copy may be in flight when the CTA exits
      mbar_wait_bounded(wbar, 0);
      for (int kk = (k >= NS ? k - NS : 0); kk < k; kk++) mbar_wait_bounded(&full[kk % NS], (kk / NS) & 1);
    }
  } else if (warp == 1) {  // ---- MMAs
    if (lane == 0) {
      bool ok = mbar_wait_bounded(wbar, 0);
      int k = 0, it = 0;
      for (int tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x, it++) {
        const int buf = it & 1;
        if (it >= 2 && !(ok = mbar_wait_bounded(&accempty[buf], ((it / 2) - 1) & 1))) break;
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(32 * buf);
        for (int t = 0; t < 9; t++, k++) {
          const int s = k % NS;
          if (!(ok = mbar_wait_bounded(&full[s], (k / NS) & 1))) break;
          tc_fence_after();
          const uint32_t a0 = smem_addr(smem + s * L::A_BYTES), b0 = smem_addr(smem + L::OFF_B + t * L::B_BYTES);
#pragma unroll
          for (int kk = 0; kk < CIN / 16; kk++)
            umma_bf16(d, umma_smem_desc(a0 + 32 * kk, L::ATOM, L::LAYOUT),
                      umma_smem_desc(b0 + 32 * kk, L::ATOM, L::LAYOUT), L::IDESC, (t | kk) != 0);
          umma_commit(&empty[s]);  // the slot is free once these MMAs have read it
        }
        if (!ok) break;
        umma_commit(&accfull[buf]);
      }
      if (!ok) atomicOr(err, 1);
      umma_commit(done);  // every MMA issued has completed once this arrives
      mbar_wait_bounded(done, 0);
    }
  } else {  // ---- epilogue: warps 2-5
    const int q = warp & 3;  // the lane quarter this warp may read
    float bv[COUT];
#pragma unroll
    for (int j = 0; j < COUT; j++) bv[j] = bias ? bias[j] : 0.f;
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, it++) {
      const int buf = it & 1;
      if (!mbar_wait_bounded(&accfull[buf], (it / 2) & 1)) {
        if (lane == 0) atomicOr(err, 1);
        break;
      }
      tc_fence_after();
      uint32_t r[COUT];
      const uint32_t src = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(32 * buf);
      tmem_ld16(src, *reinterpret_cast<uint32_t(*)[16]>(&r[0]));
      if (COUT == 32) tmem_ld16(src + 16, *reinterpret_cast<uint32_t(*)[16]>(&r[COUT == 32 ? 16 : 0]));
      tmem_wait_ld();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&accempty[buf]);  // the accumulator may take the tile after next
      const int w0 = (tile % ntw) * tw, h0 = ((tile / ntw) % nth) * th, b = tile / (ntw * nth);
      const int m = 32 * q + lane;  // this thread's accumulator lane: pixel m of the tile
      const int hh = h0 + m / tw, ww = w0 + m % tw;
      if (hh >= H || ww >= W) continue;
      const long long p = ((long long)b * H + hh) * W + ww;
      float v[COUT];
#pragma unroll
      for (int j = 0; j < COUT; j++) {
        v[j] = __uint_as_float(r[j]) + bv[j];
        if (RELU) v[j] = fmaxf(v[j], 0.f);
      }
      if (OUT_F32) {
        float4* yp = reinterpret_cast<float4*>(static_cast<float*>(y) + p * COUT);
#pragma unroll
        for (int j = 0; j < COUT / 4; j++) yp[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
      } else {
        uint4* yp = reinterpret_cast<uint4*>(static_cast<bf16*>(y) + p * COUT);
#pragma unroll
        for (int j = 0; j < COUT / 8; j++)
          yp[j] = make_uint4(pack_pair(__float2bfloat16(v[8 * j]), __float2bfloat16(v[8 * j + 1])),
                             pack_pair(__float2bfloat16(v[8 * j + 2]), __float2bfloat16(v[8 * j + 3])),
                             pack_pair(__float2bfloat16(v[8 * j + 4]), __float2bfloat16(v[8 * j + 5])),
                             pack_pair(__float2bfloat16(v[8 * j + 6]), __float2bfloat16(v[8 * j + 7])));
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 64);
  }
}

// ---------------------------------------------------------------- tcgen05 weight gradient
// dw[n][tap][c] += sum_p dy[p][n] * x[p + off(tap)][c] as tcgen05 MMAs with K = pixels:
// per 128-pixel tile, TMA loads the nine shifted x tiles (as in the forward pass) and the
// dy tile into one stage. Both operands are MN-major there (channels contiguous per
// pixel row). Four taps' x tiles, 8 KB apart, form one 128-row A operand (rows (tap, c):
// the spacing is the descriptor's leading offset), so three MMA groups -- taps 0-3, 4-7
// and 5-8 (whose last quarter, tap 8, is the one kept) -- cover the nine taps with
// M = 128, N = COUT, eight K steps of 16 pixels each. The accumulators (3 x COUT
// tensor-memory columns) sum over every tile the CTA takes; at the end the four
// epilogue warps write them to the CTA's slice of dw_part, which wgrad_reduce_kernel
// then adds to dw in CTA order (the same bits on every run).
template <int COUT>
struct TcWgrad {
  static_assert(COUT == 16 || COUT == 32, "output channels: the MMA's N");
  static constexpr int CIN = 32;
  static constexpr int A_BYTES = 128 * CIN * 2;  // one tap's x tile
  static constexpr int B_ROWB = COUT * 2;
  static constexpr int B_BYTES = 128 * B_ROWB;   // the dy tile
  static constexpr uint32_t A_LAYOUT = 4u, B_LAYOUT = COUT == 32 ? 4u : 6u;  // 64-byte / 32-byte swizzle
  static constexpr uint32_t A_SBO = 8 * CIN * 2, B_SBO = 8 * B_ROWB;
  static constexpr int STAGE = 9 * A_BYTES + B_BYTES;
  static constexpr int NST = 2;  // stages: the next tile loads while this one's MMAs run
  static constexpr int OFF_BAR = NST * STAGE;
  static constexpr int SMEM = OFF_BAR + 64 + 1024;
  static constexpr uint32_t IDESC = umma_idesc_bf16(128, COUT) | (1u << 15) | (1u << 16);  // A, B MN-major
  static constexpr int THREADS = 192;
  static_assert(STAGE % 1024 == 0 && SMEM <= 227 * 1024, "shared memory");
  // one instruction reads two 8-row K groups of four M spans of A (at most 8 KB + 2 KB past
  // its start, the last group starting at tap 5 plus seven K steps) and of one span of dy:
  // inside its stage
  static_assert(5 * A_BYTES + 14 * A_SBO + A_BYTES + 4 * A_SBO <= 9 * A_BYTES, "operand reads stay in the stage");
};

template <int COUT>
__global__ void __launch_bounds__(TcWgrad<COUT>::THREADS, 1)
    conv3x3_wgrad_tc_kernel(const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap dymap,
                            float* __restrict__ dw_part, int B, int H, int W, int tw, int th, int* err) {
  using L = TcWgrad<COUT>;
  constexpr int NST = L::NST, CIN = L::CIN;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = smem_raw + ((1024 - (smem_addr(smem_raw) & 1023)) & 1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L::OFF_BAR);
  uint64_t* empty = full + NST;
  uint64_t* accfull = empty + NST;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(accfull + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntw = (W + tw - 1) / tw, nth = (H + th - 1) / th;
  const int ntiles = B * nth * ntw;
  float* part = dw_part + (long long)blockIdx.x * COUT * 9 * CIN;  // this CTA's sums, every entry written
  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accfull, 1);
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tslot, 128);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0) {  // ---- loads
    if (lane == 0) {
      int it = 0;
      for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, it++) {
        const int s = it % NST;
        if (it >= NST && !mbar_wait_bounded(&empty[s], ((it / NST) - 1) & 1)) {
          atomicOr(err, 1);
          break;
        }
        const int w0 = (tile % ntw) * tw, h0 = ((tile / ntw) % nth) * th, b = tile / (ntw * nth);
        unsigned char* st = smem + s * L::STAGE;
        mbar_arrive_expect_tx(&full[s], L::STAGE);
        for (int t = 0; t < 9; t++) tma_load_4d(st + t * L::A_BYTES, &xmap, 0, w0 + t % 3 - 1, h0 + t / 3 - 1, b, &full[s]);
        tma_load_4d(st + 9 * L::A_BYTES, &dymap, 0, w0, h0, b, &full[s]);
      }
      for (int kk = (it >= NST ? it - NST : 0); kk < it; kk++) mbar_wait_bounded(&full[kk % NST], (kk / NST) & 1);
    }
  } else if (warp == 1) {  // ---- MMAs
    if (lane == 0) {
      bool ok = true;
      int it = 0;
      for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, it++) {
        const int s = it % NST;
        if (!(ok = mbar_wait_bounded(&full[s], (it / NST) & 1))) break;
        tc_fence_after();
        const uint32_t st = smem_addr(smem + s * L::STAGE), dy0 = st + 9 * L::A_BYTES;
#pragma unroll
        for (int g = 0; g < 3; g++) {
          const uint32_t a0 = st + (g == 0 ? 0 : (g == 1 ? 4 : 5)) * L::A_BYTES;
#pragma unroll
          for (int k = 0; k < 8; k++)  // 16 pixels = two 8-row groups per K step
            umma_bf16(tmem + (uint32_t)(g * COUT),
                      umma_smem_desc_mn(a0 + 2 * k * L::A_SBO, L::A_BYTES, L::A_SBO, L::A_LAYOUT),
                      umma_smem_desc_mn(dy0 + 2 * k * L::B_SBO, L::B_SBO, L::B_SBO, L::B_LAYOUT), L::IDESC,
                      (it | k) != 0);
        }
        umma_commit(&empty[s]);
      }
      if (!ok) atomicOr(err, 1);
      umma_commit(accfull);  // every MMA issued has completed once this arrives
    }
  } else {  // ---- epilogue: warps 2-5, once per CTA
    const int q = warp & 3;  // lane quarter: row (tap offset q within a group, c = lane)
    if (mbar_wait_bounded(accfull, 0)) {
      tc_fence_after();
#pragma unroll
      for (int g = 0; g < 3; g++) {
        if (g == 2 && q != 3) continue;  // taps 5-7 again: kept from the second group
        const int tap = (g == 0 ? 0 : (g == 1 ? 4 : 5)) + q;
#pragma unroll
        for (int n0 = 0; n0 < COUT; n0 += 16) {
          uint32_t r[16];
          tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(g * COUT + n0), r);
          tmem_wait_ld();
#pragma unroll
          for (int j = 0; j < 16; j++) part[((long long)(n0 + j) * 9 + tap) * CIN + lane] = __uint_as_float(r[j]);
        }
      }
    } else if (lane == 0) {
      atomicOr(err, 1);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, 128);
  }
}

// dw[e] += sum over the weight-gradient CTAs of their partial sums, in CTA order.
__global__ void wgrad_reduce_kernel(const float* __restrict__ part, float* __restrict__ dw, int n, int ctas) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int c = 0; c < ctas; c++) s += part[(long long)c * n + e];
    dw[e] += s;
  }
}

template <int COUT>
__global__ void bias_grad_kernel(const bf16* __restrict__ dy, float* __restrict__ db, long long P) {
  __shared__ float sh[COUT];
  for (int n = threadIdx.x; n < COUT; n += blockDim.x) sh[n] = 0.f;
  __syncthreads();
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < P * COUT; e += (long long)gridDim.x * blockDim.x)
    atomicAdd(&sh[e % COUT], __bfloat162float(dy[e]));
  __syncthreads();
  for (int n = threadIdx.x; n < COUT; n += blockDim.x) atomicAdd(&db[n], sh[n]);
}

// d[e] = (y[e] > 0) ? d[e] : 0   (ReLU backward through the post-activation output y)
__global__ void relu_back_kernel(bf16* __restrict__ d, const bf16* __restrict__ y, long long n) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    if (!(__bfloat162float(y[e]) > 0.f)) d[e] = __float2bfloat16(0.f);
}

// wT[c][tap][n] = w[n][8 - tap][c]: the weights of the input-gradient convolution.
__global__ void flip_weights_kernel(const bf16* __restrict__ w, bf16* __restrict__ wT, int cin, int cout) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= cin * 9 * cout) return;
  const int n = e % cout, tap = (e / cout) % 9, c = e / (cout * 9);
  wT[e] = w[((long long)n * 9 + (8 - tap)) * cin + c];
}

// x16[p][c] = c < 24 ? bf16(x[p][c]) : 0, c < 32
__global__ void pack_input_kernel(const float* __restrict__ x, bf16* __restrict__ x16, long long P) {
  constexpr int CP = kCin[0];
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < P * CP; e += (long long)gridDim.x * blockDim.x) {
    const long long p = e / CP;
    const int c = (int)(e % CP);
    x16[e] = __float2bfloat16(c < kInReal ? x[p * kInReal + c] : 0.f);
  }
}

// out3[p][c] = out16[p][c], c < 3
__global__ void unpack_output_kernel(const float* __restrict__ out16, float* __restrict__ out3, long long P) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < P * kOutReal;
       e += (long long)gridDim.x * blockDim.x)
    out3[e] = out16[(e / kOutReal) * 16 + e % kOutReal];
}

// Mean squared error over the 3 real channels; gradient (bf16, 16 channels) and the loss sum.
__global__ void mse_kernel(const float* __restrict__ out16, const float* __restrict__ target, bf16* __restrict__ d16,
                           float* __restrict__ loss, long long P) {
  __shared__ float sh[256];
  float s = 0.f;
  const float scale = 2.f / (float)(P * kOutReal);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < P * 16; e += (long long)gridDim.x * blockDim.x) {
    const long long p = e / 16;
    const int c = (int)(e % 16);
    float g = 0.f;
    if (c < kOutReal) {
      const float r = out16[e] - target[p * kOutReal + c];
      s += r * r;
      g = scale * r;
    }
    d16[e] = __float2bfloat16(g);
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, sh[0]);
}

// Adam on FP32 master parameters; writes the BF16 copy used by the kernels.
__global__ void adam_kernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                            const float* __restrict__ g, bf16* __restrict__ p16, int n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float gg = g[e];
  const float mm = b1 * m[e] + (1.f - b1) * gg;
  const float vv = b2 * v[e] + (1.f - b2) * gg * gg;
  m[e] = mm;
  v[e] = vv;
  const float upd = lr * (mm / c1) / (sqrtf(vv / c2) + eps);
  p[e] -= upd;
  if (p16) p16[e] = __float2bfloat16(p[e]);
}

__global__ void f32_to_bf16_kernel(const float* __restrict__ a, bf16* __restrict__ b, int n) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) b[e] = __float2bfloat16(a[e]);
}

// Features of a layered wave state (AoS FP64 u, v, p on ny = blocks x block_rows
// rows of nx points) for the network. In the impedance-scaled variables
// q = (Z u, Z v, p), Z = sqrt(rho K), the coarse solve's error does not depend
// on the layer away from the interface (equal wave speeds). Per point, divided
// by the feature scale s (inv_scale = 1/s):
//   x[0..2]   = d2x q    undivided second differences along x,
//   x[3..5]   = d2y q    along y, within the point's block (no differencing
//                        across the interface line, which both blocks hold),
//   x[6..8]   = d4x q    undivided fourth differences along x,
//   x[9..11]  = d4y q    along y, within the block,
//   x[12..23] = t x[0..11]   t = +1 in block 0, -1 above (the layer tag),
// with each centre clamped one (two, for d4) point(s) in from an edge, so the
// difference is one-sided there. The differences are taken in FP64 before the
// network's BF16 rounding. The features are high-pass and linear in the state;
// the network's ReLU layers without biases are positively homogeneous, so a
// smooth or zero state gets a proportionally small or zero correction.
__device__ __forceinline__ void zq(const double* __restrict__ state, const double* __restrict__ rho,
                                   const double* __restrict__ K, long long p, double (&q)[3]) {
  const double z = sqrt(rho[p] * K[p]);
  q[0] = z * state[3 * p + 0];
  q[1] = z * state[3 * p + 1];
  q[2] = state[3 * p + 2];
}

// Second (D4 = false) or fourth (D4 = true) undivided difference of q at point p0 with stride st.
template <bool D4>
__device__ __forceinline__ void diff_q(const double* __restrict__ state, const double* __restrict__ rho,
                                       const double* __restrict__ K, long long p0, long long st, double (&d)[3]) {
  double a[3], b[3], m[3];
  zq(state, rho, K, p0, m);
  if (!D4) {
    zq(state, rho, K, p0 - st, a);
    zq(state, rho, K, p0 + st, b);
    for (int c = 0; c < 3; c++) d[c] = a[c] - 2.0 * m[c] + b[c];
  } else {
    double a2[3], b2[3];
    zq(state, rho, K, p0 - 2 * st, a2);
    zq(state, rho, K, p0 - st, a);
    zq(state, rho, K, p0 + st, b);
    zq(state, rho, K, p0 + 2 * st, b2);
    for (int c = 0; c < 3; c++) d[c] = a2[c] - 4.0 * a[c] + 6.0 * m[c] - 4.0 * b[c] + b2[c];
  }
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__global__ void features_kernel(const double* __restrict__ state, const double* __restrict__ rho,
                                const double* __restrict__ K, float* __restrict__ x, int nx, int ny, int block_rows,
                                double inv_scale) {
  const long long P = (long long)nx * ny;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(p / nx), i = (int)(p % nx);
    const int b = j / block_rows, r = j % block_rows;
    const long long row0 = (long long)b * block_rows;
    double f[12], d[3];
    diff_q<false>(state, rho, K, (long long)j * nx + clampi(i, 1, nx - 2), 1, d);
    for (int c = 0; c < 3; c++) f[c] = d[c];
    diff_q<false>(state, rho, K, (row0 + clampi(r, 1, block_rows - 2)) * nx + i, nx, d);
    for (int c = 0; c < 3; c++) f[3 + c] = d[c];
    diff_q<true>(state, rho, K, (long long)j * nx + clampi(i, 2, nx - 3), 1, d);
    for (int c = 0; c < 3; c++) f[6 + c] = d[c];
    diff_q<true>(state, rho, K, (row0 + clampi(r, 2, block_rows - 3)) * nx + i, nx, d);
    for (int c = 0; c < 3; c++) f[9 + c] = d[c];
    const double t = b == 0 ? 1.0 : -1.0;
    for (int c = 0; c < 12; c++) {
      x[(long long)kInReal * p + c] = (float)(f[c] * inv_scale);
      x[(long long)kInReal * p + 12 + c] = (float)(t * f[c] * inv_scale);
    }
  }
}

// The network's output is a correction of q = (Z u, Z v, p) in units of `scale`:
// state[p] += scale * (delta[p][0] / Z, delta[p][1] / Z, delta[p][2]).
__global__ void correct_kernel(double* __restrict__ state, const float* __restrict__ delta,
                               const double* __restrict__ rho, const double* __restrict__ K, long long P,
                               double scale) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
    const double zi = scale / sqrt(rho[p] * K[p]);
    state[3 * p + 0] += zi * (double)delta[3 * p + 0];
    state[3 * p + 1] += zi * (double)delta[3 * p + 1];
    state[3 * p + 2] += scale * (double)delta[3 * p + 2];
  }
}

inline int blocks_for(long long n, int threads) {
  long long b = (n + threads - 1) / threads;
  return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
}

}  // namespace cnn
}  // namespace sbp

using namespace sbp::cnn;

struct sbp_cnn {
  int H = 0, W = 0, maxB = 0, device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  long long step = 0;
  float* wm[kLayers] = {};   // FP32 master weights [cout][9][cin]
  bf16* wb[kLayers] = {};    // BF16 copies
  bf16* wT[kLayers] = {};    // flipped, transposed (input-gradient) weights
  float* bias[kLayers] = {};
  float *mw[kLayers] = {}, *vw[kLayers] = {}, *mbias[kLayers] = {}, *vbias[kLayers] = {};
  float *gw[kLayers] = {}, *gb[kLayers] = {};
  bf16* act[kLayers] = {};   // layer inputs: act[0] = packed input, act[l] = output of layer l-1
  bf16* dact = nullptr;      // gradient buffers (two, ping-pong)
  bf16* dact2 = nullptr;
  float* out16 = nullptr;    // last layer output (FP32, 16 channels)
  float* loss = nullptr;
  int* err = nullptr;        // the tensor-core convolutions' error word (a bounded wait ran out)
  int tw = 0, th = 0;        // their pixel tile: th rows of tw pixels, th * tw = 128
  int nsm = 1;               // SMs: the persistent convolutions' grid
  float* dw_part = nullptr;  // the weight gradient's per-CTA sums ([nsm][32 * 9 * 32])
  long long launches = 0;
  std::string msg;
};

namespace {

thread_local std::string g_cnn_error;

int cfail(sbp_cnn* c, int code, const std::string& m) {
  if (c) c->msg = m;
  else g_cnn_error = m;
  return code;
}

#define CCK(call)                                                                        \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return cfail(c, SBP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

long long wcount(int l) { return (long long)kCout[l] * 9 * kCin[l]; }

void cnn_release(sbp_cnn* c) {
  for (int l = 0; l < kLayers; l++) {
    void* ps[] = {c->wm[l], c->wb[l], c->wT[l], c->bias[l], c->mw[l], c->vw[l], c->mbias[l], c->vbias[l],
                  c->gw[l], c->gb[l], c->act[l]};
    for (void* p : ps)
      if (p) cudaFree(p);
  }
  void* ps[] = {c->dact, c->dact2, c->out16, c->loss, c->err, c->dw_part};
  for (void* p : ps)
    if (p) cudaFree(p);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// The tensor maps of one convolution: the NHWC BF16 input ({ch, W, H, B}, box {ch, tw,
// th, 1}) and the weights ([cout][9][ch]: {ch, 9, cout}, box {ch, 1, cout}), rows
// swizzled over their ch * 2 bytes. Out-of-range boxes read zeros (the image border).
cudaError_t encode_conv_maps(const sbp_cnn* c, const bf16* x, const bf16* w, int ch, int cout, int batch,
                             CUtensorMap* xm, CUtensorMap* wm) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  const CUtensorMapSwizzle sw = ch == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B;
  const cuuint64_t xd[4] = {(cuuint64_t)ch, (cuuint64_t)c->W, (cuuint64_t)c->H, (cuuint64_t)batch};
  const cuuint64_t xs[3] = {(cuuint64_t)ch * 2, (cuuint64_t)c->W * ch * 2, (cuuint64_t)c->H * c->W * ch * 2};
  const cuuint32_t xb[4] = {(cuuint32_t)ch, (cuuint32_t)c->tw, (cuuint32_t)c->th, 1};
  const cuuint32_t e[4] = {1, 1, 1, 1};
  if (enc(xm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16*>(x), xd, xs, xb, e, CU_TENSOR_MAP_INTERLEAVE_NONE,
          sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  const cuuint64_t wd[3] = {(cuuint64_t)ch, 9, (cuuint64_t)cout};
  const cuuint64_t ws[2] = {(cuuint64_t)ch * 2, (cuuint64_t)9 * ch * 2};
  const cuuint32_t wbx[3] = {(cuuint32_t)ch, 1, (cuuint32_t)cout};
  if (enc(wm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<bf16*>(w), wd, ws, wbx, e, CU_TENSOR_MAP_INTERLEAVE_NONE,
          sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return cudaErrorInvalidValue;
  return cudaSuccess;
}

template <int CIN, int COUT, bool RELU, bool OUT_F32>
cudaError_t configure_tc() {
  return cudaFuncSetAttribute(conv3x3_tc_kernel<CIN, COUT, RELU, OUT_F32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              TcConv<CIN, COUT>::SMEM);
}

template <int CIN, int COUT, bool RELU, bool OUT_F32>
cudaError_t launch_tc(const bf16* x, const bf16* w, const float* bias, void* y, const sbp_cnn* c, int batch,
                      cudaStream_t s) {
  CUtensorMap xm, wm;
  cudaError_t e = encode_conv_maps(c, x, w, CIN, COUT, batch, &xm, &wm);
  if (e != cudaSuccess) return e;
  const long long tiles = (long long)batch * ((c->H + c->th - 1) / c->th) * ((c->W + c->tw - 1) / c->tw);
  const long long slots = (long long)TcConv<CIN, COUT>::CTAS * c->nsm;  // persistent: every CTA resident
  const unsigned grid = (unsigned)(tiles < slots ? tiles : slots);
  conv3x3_tc_kernel<CIN, COUT, RELU, OUT_F32><<<grid, TcConv<CIN, COUT>::THREADS, TcConv<CIN, COUT>::SMEM, s>>>(
      xm, wm, bias, y, batch, c->H, c->W, c->tw, c->th, c->err);
  return cudaGetLastError();
}

template <int COUT>
cudaError_t configure_wgrad_tc() {
  return cudaFuncSetAttribute(conv3x3_wgrad_tc_kernel<COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              TcWgrad<COUT>::SMEM);
}

// Shared-memory opt-in of the tensor-core convolutions (outside stream capture).
cudaError_t configure_convs() {
  cudaError_t e;
  if ((e = configure_tc<32, 32, true, false>()) != cudaSuccess) return e;
  if ((e = configure_tc<32, 16, false, true>()) != cudaSuccess) return e;
  if ((e = configure_tc<32, 32, false, false>()) != cudaSuccess) return e;
  if ((e = configure_tc<16, 32, false, false>()) != cudaSuccess) return e;
  if ((e = configure_wgrad_tc<32>()) != cudaSuccess) return e;
  return configure_wgrad_tc<16>();
}

// Launch one conv of layer l (forward) or its input-gradient conv.
cudaError_t conv_fwd(int l, const bf16* x, void* y, const sbp_cnn* c, int batch, cudaStream_t s) {
  if (l < kLayers - 1) return launch_tc<32, 32, true, false>(x, c->wb[l], c->bias[l], y, c, batch, s);
  return launch_tc<32, 16, false, true>(x, c->wb[l], c->bias[l], y, c, batch, s);
}

cudaError_t conv_dgrad(int l, const bf16* dy, bf16* dx, const sbp_cnn* c, int batch, cudaStream_t s) {
  if (l == kLayers - 1) return launch_tc<16, 32, false, false>(dy, c->wT[l], nullptr, dx, c, batch, s);
  return launch_tc<32, 32, false, false>(dy, c->wT[l], nullptr, dx, c, batch, s);
}

// dw += the weight gradient of layer l (x: its input, 32 channels; dy: its output gradient).
cudaError_t conv_wgrad(int l, const bf16* x, const bf16* dy, float* dw, const sbp_cnn* c, int batch, cudaStream_t s) {
  CUtensorMap xm, dym, unused;
  const int cout = kCout[l];
  // x: 32-channel tap tiles; dy: one unshifted tile of cout channels (its map from the same
  // encoder, with dy as the "input" and the weights map unused)
  cudaError_t e = encode_conv_maps(c, x, c->wb[l], 32, cout, batch, &xm, &unused);
  if (e == cudaSuccess) e = encode_conv_maps(c, dy, c->wb[l], cout, cout, batch, &dym, &unused);
  if (e != cudaSuccess) return e;
  const long long tiles = (long long)batch * ((c->H + c->th - 1) / c->th) * ((c->W + c->tw - 1) / c->tw);
  const unsigned grid = (unsigned)(tiles < c->nsm ? tiles : c->nsm);
  if (cout == 32)
    conv3x3_wgrad_tc_kernel<32><<<grid, TcWgrad<32>::THREADS, TcWgrad<32>::SMEM, s>>>(
        xm, dym, c->dw_part, batch, c->H, c->W, c->tw, c->th, c->err);
  else
    conv3x3_wgrad_tc_kernel<16><<<grid, TcWgrad<16>::THREADS, TcWgrad<16>::SMEM, s>>>(
        xm, dym, c->dw_part, batch, c->H, c->W, c->tw, c->th, c->err);
  const int n = (int)wcount(l);
  wgrad_reduce_kernel<<<(n + 255) / 256, 256, 0, s>>>(c->dw_part, dw, n, (int)grid);
  return cudaGetLastError();
}

cudaError_t bias_grad(int l, const bf16* dy, float* db, int batch, const sbp_cnn* c, cudaStream_t s) {
  const long long P = (long long)batch * c->H * c->W;
  if (kCout[l] == 32)
    bias_grad_kernel<32><<<blocks_for(P * 32, 256), 256, 0, s>>>(dy, db, P);
  else
    bias_grad_kernel<16><<<blocks_for(P * 16, 256), 256, 0, s>>>(dy, db, P);
  return cudaGetLastError();
}

int refresh_weights(sbp_cnn* c) {
  for (int l = 0; l < kLayers; l++) {
    const int n = (int)wcount(l);
    f32_to_bf16_kernel<<<(n + 255) / 256, 256, 0, c->stream>>>(c->wm[l], c->wb[l], n);
    flip_weights_kernel<<<(n + 255) / 256, 256, 0, c->stream>>>(c->wb[l], c->wT[l], kCin[l], kCout[l]);
    c->launches += 2;
  }
  CCK(cudaGetLastError());
  return SBP_OK;
}

int run_forward(sbp_cnn* c, const float* x, int batch) {
  const long long P = (long long)batch * c->H * c->W;
  pack_input_kernel<<<blocks_for(P * kCin[0], 256), 256, 0, c->stream>>>(x, c->act[0], P);
  c->launches++;
  for (int l = 0; l < kLayers; l++) {
    void* y = (l == kLayers - 1) ? (void*)c->out16 : (void*)c->act[l + 1];
    CCK(conv_fwd(l, c->act[l], y, c, batch, c->stream));
    c->launches++;
  }
  return SBP_OK;
}

// Masks that keep padded channels of parameters at zero (never trained).
bool weight_is_real(int l, long long e) {
  const int cin = kCin[l];
  const int ci = (int)(e % cin);
  const int n = (int)(e / (9LL * cin));
  if (l == 0 && ci >= kInReal) return false;
  if (l == kLayers - 1 && n >= kOutReal) return false;
  return true;
}

}  // namespace

extern "C" {

int sbp_cnn_create(int height, int width, int max_batch, int device, void* stream, sbp_cnn** out) {
  if (!out || height < 1 || width < 1 || max_batch < 1) return cfail(nullptr, SBP_ERR_INVALID, "bad network size");
  *out = nullptr;
  sbp_cnn* c = new (std::nothrow) sbp_cnn();
  if (!c) return cfail(nullptr, SBP_ERR_INVALID, "out of host memory");
  c->H = height;
  c->W = width;
  c->maxB = max_batch;
  c->device = device;
  auto bad = [&](const std::string& m) {
    g_cnn_error = m;
    cnn_release(c);
    delete c;
    return SBP_ERR_CUDA;
  };
  if (cudaSetDevice(device) != cudaSuccess) return bad("cudaSetDevice failed");
  if (stream) {
    c->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return bad("stream");
    c->own_stream = true;
  }
  const long long P = (long long)max_batch * height * width;
  for (int l = 0; l < kLayers; l++) {
    const size_t nw = (size_t)wcount(l), nb = (size_t)kCout[l];
    if (cudaMalloc(&c->wm[l], nw * 4) || cudaMalloc(&c->wb[l], nw * 2) || cudaMalloc(&c->wT[l], nw * 2) ||
        cudaMalloc(&c->bias[l], nb * 4) || cudaMalloc(&c->mw[l], nw * 4) || cudaMalloc(&c->vw[l], nw * 4) ||
        cudaMalloc(&c->mbias[l], nb * 4) || cudaMalloc(&c->vbias[l], nb * 4) || cudaMalloc(&c->gw[l], nw * 4) ||
        cudaMalloc(&c->gb[l], nb * 4) || cudaMalloc(&c->act[l], (size_t)P * kCin[l] * 2))
      return bad("cudaMalloc(network)");
    cudaMemset(c->mw[l], 0, nw * 4);
    cudaMemset(c->vw[l], 0, nw * 4);
    cudaMemset(c->mbias[l], 0, nb * 4);
    cudaMemset(c->vbias[l], 0, nb * 4);
  }
  if (cudaMalloc(&c->dact, (size_t)P * 32 * 2) || cudaMalloc(&c->dact2, (size_t)P * 32 * 2) ||
      cudaMalloc(&c->out16, (size_t)P * 16 * 4) || cudaMalloc(&c->loss, 4) || cudaMalloc(&c->err, 4))
    return bad("cudaMalloc(activations)");
  cudaMemset(c->err, 0, 4);
  // the tensor-core convolutions' tile: 128 pixels, th rows of tw (a power of two), the
  // shape whose tiles cover the image with the fewest padding pixels (ties: wider rows)
  long long best = -1;
  for (int tw = 128; tw >= 1; tw /= 2) {
    const int th = 128 / tw;
    const long long area = (long long)((width + tw - 1) / tw) * tw * ((height + th - 1) / th) * th;
    if (best < 0 || area < best) {
      best = area;
      c->tw = tw;
      c->th = th;
    }
  }
  if (configure_convs() != cudaSuccess) return bad("cudaFuncSetAttribute(convolutions)");
  if (cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || c->nsm < 1)
    return bad("cudaDeviceGetAttribute(SMs)");
  if (cudaMalloc(&c->dw_part, (size_t)c->nsm * 32 * 9 * 32 * sizeof(float)) != cudaSuccess)
    return bad("cudaMalloc(weight-gradient partial sums)");
  if (!encode_fn()) return bad("cuTensorMapEncodeTiled is not available from the driver");
  // a network that failed its initialisation is released, not handed out
  const int rc = sbp_cnn_init(c, 1234);
  if (rc) {
    g_cnn_error = c->msg;
    cnn_release(c);
    delete c;
    return rc;
  }
  *out = c;
  return SBP_OK;
}

int sbp_cnn_destroy(sbp_cnn* c) {
  if (!c) return SBP_ERR_INVALID;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  cnn_release(c);
  delete c;
  return SBP_OK;
}

const char* sbp_cnn_last_error(const sbp_cnn* c) { return c ? c->msg.c_str() : g_cnn_error.c_str(); }

long long sbp_cnn_param_count(void) {
  long long n = 0;
  for (int l = 0; l < kLayers; l++) n += wcount(l) + kCout[l];
  return n;
}

int sbp_cnn_init(sbp_cnn* c, unsigned long long seed) {
  if (!c) return SBP_ERR_INVALID;
  CCK(cudaSetDevice(c->device));
  std::mt19937_64 rng(seed);
  for (int l = 0; l < kLayers; l++) {
    const long long n = wcount(l);
    const int fan_in = 9 * (l == 0 ? kInReal : kCin[l]);
    // He-normal hidden layers; the output layer starts at zero, so the untrained network is the
    // zero correction and training moves away from it only where that lowers the error.
    std::normal_distribution<double> nd(0.0, std::sqrt(2.0 / fan_in) * (l == kLayers - 1 ? 0.0 : 1.0));
    std::vector<float> w(n);
    for (long long e = 0; e < n; e++) w[e] = weight_is_real(l, e) ? (float)nd(rng) : 0.f;
    std::vector<float> b(kCout[l], 0.f);
    CCK(cudaMemcpyAsync(c->wm[l], w.data(), n * 4, cudaMemcpyHostToDevice, c->stream));
    CCK(cudaMemcpyAsync(c->bias[l], b.data(), b.size() * 4, cudaMemcpyHostToDevice, c->stream));
    CCK(cudaMemsetAsync(c->mw[l], 0, n * 4, c->stream));
    CCK(cudaMemsetAsync(c->vw[l], 0, n * 4, c->stream));
    CCK(cudaMemsetAsync(c->mbias[l], 0, kCout[l] * 4, c->stream));
    CCK(cudaMemsetAsync(c->vbias[l], 0, kCout[l] * 4, c->stream));
  }
  c->step = 0;
  int rc = refresh_weights(c);
  if (rc) return rc;
  CCK(cudaStreamSynchronize(c->stream));
  return SBP_OK;
}

// Parameters as one FP32 vector: per layer, weights [cout][9][cin] then bias [cout].
int sbp_cnn_get_params(sbp_cnn* c, float* host, long long n) {
  if (!c || !host || n != sbp_cnn_param_count()) return SBP_ERR_INVALID;
  CCK(cudaSetDevice(c->device));
  long long o = 0;
  for (int l = 0; l < kLayers; l++) {
    CCK(cudaMemcpyAsync(host + o, c->wm[l], wcount(l) * 4, cudaMemcpyDeviceToHost, c->stream));
    o += wcount(l);
    CCK(cudaMemcpyAsync(host + o, c->bias[l], kCout[l] * 4, cudaMemcpyDeviceToHost, c->stream));
    o += kCout[l];
  }
  CCK(cudaStreamSynchronize(c->stream));
  return SBP_OK;
}

int sbp_cnn_set_params(sbp_cnn* c, const float* host, long long n) {
  if (!c || !host || n != sbp_cnn_param_count()) return SBP_ERR_INVALID;
  CCK(cudaSetDevice(c->device));
  long long o = 0;
  for (int l = 0; l < kLayers; l++) {
    CCK(cudaMemcpyAsync(c->wm[l], host + o, wcount(l) * 4, cudaMemcpyHostToDevice, c->stream));
    o += wcount(l);
    CCK(cudaMemcpyAsync(c->bias[l], host + o, kCout[l] * 4, cudaMemcpyHostToDevice, c->stream));
    o += kCout[l];
  }
  int rc = refresh_weights(c);
  if (rc) return rc;
  CCK(cudaStreamSynchronize(c->stream));
  return SBP_OK;
}

// out = network(x): x, out device arrays, NHWC FP32, 4 and 3 channels.
int sbp_cnn_forward(sbp_cnn* c, const float* x, int batch, float* out) {
  if (!c || !x || !out || batch < 1 || batch > c->maxB) return SBP_ERR_INVALID;
  CCK(cudaSetDevice(c->device));
  int rc = run_forward(c, x, batch);
  if (rc) return rc;
  const long long P = (long long)batch * c->H * c->W;
  unpack_output_kernel<<<blocks_for(P * 3, 256), 256, 0, c->stream>>>(c->out16, out, P);
  c->launches++;
  int e = 0;
  CCK(cudaMemcpyAsync(&e, c->err, 4, cudaMemcpyDeviceToHost, c->stream));
  CCK(cudaStreamSynchronize(c->stream));
  if (e) {
    CCK(cudaMemsetAsync(c->err, 0, 4, c->stream));
    return cfail(c, SBP_ERR_DEVICE, "a tensor-core convolution's wait for its tiles ran out");
  }
  return SBP_OK;
}

// Gradients of the mean squared error of network(x) against target (both device, NHWC FP32,
// 4 and 3 channels), without updating the parameters; written as one FP32 vector in the
// layout of sbp_cnn_get_params (host `grad`, may be NULL). Returns the loss in *loss.
// bias_grads: also the biases' gradients (the training step leaves biases untrained and skips them).
static int backward(sbp_cnn* c, const float* x, const float* target, int batch, float* loss, bool bias_grads) {
  const long long P = (long long)batch * c->H * c->W;
  int rc = run_forward(c, x, batch);
  if (rc) return rc;
  CCK(cudaMemsetAsync(c->loss, 0, 4, c->stream));
  mse_kernel<<<blocks_for(P * 16, 256), 256, 0, c->stream>>>(c->out16, target, c->dact, c->loss, P);
  c->launches++;
  for (int l = 0; l < kLayers; l++) {
    CCK(cudaMemsetAsync(c->gw[l], 0, wcount(l) * 4, c->stream));
    CCK(cudaMemsetAsync(c->gb[l], 0, kCout[l] * 4, c->stream));
  }
  bf16* dcur = c->dact;   // gradient w.r.t. the output of layer l (pre-activation once masked)
  bf16* dnext = c->dact2;
  for (int l = kLayers - 1; l >= 0; l--) {
    CCK(conv_wgrad(l, c->act[l], dcur, c->gw[l], c, batch, c->stream));
    c->launches += 2;  // weight gradient and its reduction
    if (bias_grads) {
      CCK(bias_grad(l, dcur, c->gb[l], batch, c, c->stream));
      c->launches++;
    }
    if (l == 0) break;
    CCK(conv_dgrad(l, dcur, dnext, c, batch, c->stream));
    relu_back_kernel<<<blocks_for(P * kCin[l], 256), 256, 0, c->stream>>>(dnext, c->act[l], P * kCin[l]);
    c->launches += 2;
    bf16* tmp = dcur;
    dcur = dnext;
    dnext = tmp;
  }
  float h = 0;
  int e = 0;
  CCK(cudaMemcpyAsync(&h, c->loss, 4, cudaMemcpyDeviceToHost, c->stream));
  CCK(cudaMemcpyAsync(&e, c->err, 4, cudaMemcpyDeviceToHost, c->stream));
  CCK(cudaStreamSynchronize(c->stream));
  if (e) {
    CCK(cudaMemsetAsync(c->err, 0, 4, c->stream));
    return cfail(c, SBP_ERR_DEVICE, "a tensor-core convolution's wait for its tiles ran out");
  }
  if (loss) *loss = h / (float)(P * kOutReal);
  return SBP_OK;
}

int sbp_cnn_gradients(sbp_cnn* c, const float* x, const float* target, int batch, float* grad, long long n,
                      float* loss) {
  if (!c || !x || !target || batch < 1 || batch > c->maxB) return SBP_ERR_INVALID;
  if (grad && n != sbp_cnn_param_count()) return SBP_ERR_INVALID;
  CCK(cudaSetDevice(c->device));
  int rc = backward(c, x, target, batch, loss, true);
  if (rc || !grad) return rc;
  long long o = 0;
  for (int l = 0; l < kLayers; l++) {
    CCK(cudaMemcpyAsync(grad + o, c->gw[l], wcount(l) * 4, cudaMemcpyDeviceToHost, c->stream));
    o += wcount(l);
    CCK(cudaMemcpyAsync(grad + o, c->gb[l], kCout[l] * 4, cudaMemcpyDeviceToHost, c->stream));
    o += kCout[l];
  }
  CCK(cudaStreamSynchronize(c->stream));
  return SBP_OK;
}

// One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the mean squared error.
// Weights are trained; biases keep their values (zero from sbp_cnn_init), so
// the trained network maps zero features to zero outputs.
int sbp_cnn_train_step(sbp_cnn* c, const float* x, const float* target, int batch, float lr, float* loss) {
  if (!c || !x || !target || batch < 1 || batch > c->maxB || !(lr > 0)) return SBP_ERR_INVALID;
  CCK(cudaSetDevice(c->device));
  int rc = backward(c, x, target, batch, loss, false);
  if (rc) return rc;
  c->step++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)c->step), c2 = 1.f - std::pow(b2, (float)c->step);
  for (int l = 0; l < kLayers; l++) {
    const int n = (int)wcount(l);
    adam_kernel<<<(n + 255) / 256, 256, 0, c->stream>>>(c->wm[l], c->mw[l], c->vw[l], c->gw[l], nullptr, n, lr, b1, b2,
                                                        1e-8f, c1, c2);
    c->launches += 1;
  }
  // padded channels stay zero: their gradients are zero (zero inputs / zero targets) and
  // Adam leaves zero-gradient entries unchanged.
  rc = refresh_weights(c);
  if (rc) return rc;
  CCK(cudaStreamSynchronize(c->stream));
  return SBP_OK;
}

int sbp_cnn_features(const double* state, const double* rho, const double* K, int nx, int ny, int block_rows,
                     double inv_scale, float* x, void* stream) {
  if (!state || !rho || !K || !x || nx < 5 || block_rows < 5 || ny < block_rows || ny % block_rows)
    return SBP_ERR_INVALID;
  const long long P = (long long)nx * ny;
  features_kernel<<<blocks_for(P, 256), 256, 0, (cudaStream_t)stream>>>(state, rho, K, x, nx, ny, block_rows,
                                                                        inv_scale);
  return cudaGetLastError() == cudaSuccess ? SBP_OK : SBP_ERR_CUDA;
}

int sbp_cnn_correct(double* state, const float* delta, const double* rho, const double* K, long long npts,
                    double scale, void* stream) {
  if (!state || !delta || !rho || !K || npts < 1) return SBP_ERR_INVALID;
  correct_kernel<<<blocks_for(npts, 256), 256, 0, (cudaStream_t)stream>>>(state, delta, rho, K, npts, scale);
  return cudaGetLastError() == cudaSuccess ? SBP_OK : SBP_ERR_CUDA;
}

long long sbp_cnn_launch_count(const sbp_cnn* c) { return c ? c->launches : SBP_ERR_INVALID; }

}  // extern "C"
