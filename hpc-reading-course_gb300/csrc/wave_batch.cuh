// wave_batch.cuh -- many independent wave / advection instances of uneven
// size, order and coefficients advanced together.
//
// Wave instances (rho = 1, K = c^2, one constant per instance) run through a
// persistent stage kernel per operator order: its grid walks a tile list of
// (instance, tile) pairs. The producer warp loads each tile's state tiles
// with TMA from the instance's own tensor maps (kept in global memory) and
// bulk-copies the instance's parameter block (taps, SAT weights, pointers,
// time step) into the same shared-memory stage, so consumers read every
// per-instance constant from shared memory. The per-tile arithmetic is the
// single-instance kernel's (wave_tile_compute).
//
// Advection instances (one component) use one CTA per (instance, tile) pair;
// their per-point arithmetic is the single-instance line kernel's.
#pragma once

#include "line_kernels.cuh"
#include "wave2d.cuh"

namespace sbp {

// Per-instance block of a batched wave instance; 16-byte multiple so it can
// be bulk-copied into shared memory.
template <typename T> struct alignas(16) BatchWave {
  WaveParams<T> prm;  // geometry, taps, SAT weights, kconst, dt, un/acc/comp pointers
  T* wa;              // stage-input ping-pong buffers
  T* wb;
  T c_acc[4], c_w[4];  // RK4 stage rk's coefficients at [rk - 1], computed on the host
};

// Tensor maps of one batched wave instance, in global memory (64-byte aligned):
// [3 * s + {0,1,2}] = stage input s (0: u^n, 1: wa, 2: wb) with the p, u, v
// tile boxes; [9], [10], [11] = u^n, acc, comp point boxes.
constexpr int kBatchMaps = 12;

// Stage input and output buffers and RK4 coefficients of stage rk (1..4) of
// the classical RK4 step sequence (see the single-instance runtime). The
// coefficients come from the instance block: computing dt / 6 here would put an
// FP64 division per tile and thread on the FP64 pipe, which the FP32 kernels
// otherwise barely use (measured: it held the pipe 58-64 % busy).
template <typename T>
__device__ __forceinline__ void batch_stage_buffers(const BatchWave<T>& I, int rk, const T*& in, T*& wout, T& c_acc,
                                                    T& c_w) {
  in = rk == 1 ? I.prm.un : (rk == 3 ? I.wb : I.wa);
  wout = (rk == 1 || rk == 3) ? I.wa : I.wb;
  c_acc = I.c_acc[rk - 1];
  c_w = I.c_w[rk - 1];
}

// acc coefficients dt / 6, dt / 3, dt / 3, dt / 6 and stage-input coefficients
// dt / 2, dt / 2, dt (the last stage has none) in the state type, rounded as the
// single-instance runtime rounds them.
template <typename T> inline void batch_rk4_coefficients(double dt, T (&c_acc)[4], T (&c_w)[4]) {
  for (int rk = 1; rk <= 4; rk++) {
    c_acc[rk - 1] = (T)((rk == 1 || rk == 4) ? dt / 6 : dt / 3);
    c_w[rk - 1] = (T)(rk == 3 ? dt : 0.5 * dt);
  }
}

// A tile-list entry: the instance's slot and the tile's origin, so the
// producer issues its loads without first reading the instance block.
struct BatchTile {
  int slot, i0, j0, pad;
};

// Consumer warps of the batched wave kernel per precision.
#ifndef SBP_BATCH_WARPS_F32
#define SBP_BATCH_WARPS_F32 16
#endif
#ifndef SBP_BATCH_WARPS_F64
#define SBP_BATCH_WARPS_F64 8
#endif
template <typename T> constexpr int batch_warps() { return sizeof(T) == 4 ? SBP_BATCH_WARPS_F32 : SBP_BATCH_WARPS_F64; }
template <typename T, int ORD, int STAGE, int TY>
using BatchWaveTile = WaveTile<T, ORD, STAGE, TY, (int)sizeof(BatchWave<T>), false, 2, batch_warps<T>()>;

// A CTA takes every gridDim.x-th tile of the list, so neighbouring tiles of an
// instance run at the same time on neighbouring CTAs and share their halo rows in
// L2. Measured at 512 instances: contiguous ranges of the list per CTA ran at
// 1.39e10 (FP64) / 2.36e10 (FP32) point-stage updates/s against 1.72e10 / 3.22e10,
// and prefetching the next instance's tensor maps changed nothing.
template <typename T, int ORD, int STAGE, int TY>
__global__ void __launch_bounds__(BatchWaveTile<T, ORD, STAGE, TY>::THREADS, 1)
    wave_batch_stage_kernel(const BatchWave<T>* __restrict__ insts, const CUtensorMap* __restrict__ maps,
                            const BatchTile* __restrict__ tiles, int ntiles, int rk, int* err) {
  using Tile = BatchWaveTile<T, ORD, STAGE, TY>;
  constexpr int HX = Tile::HX, HY = Tile::HY;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + Tile::OFF_BAR);
  uint64_t* empty = full + 2;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  uint64_t* dbar = reinterpret_cast<uint64_t*>(smem + Tile::OFF_DBAR);
  if (threadIdx.x == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    mbar_init(&empty[0], Tile::WARPS);
    mbar_init(&empty[1], Tile::WARPS);
    mbar_init(&dbar[0], Tile::WARPS);
    mbar_init(&dbar[1], Tile::WARPS);
    fence_barrier_init();
  }
  __syncthreads();
  const int sel = rk == 1 ? 0 : (rk == 3 ? 2 : 1);  // which buffer is the stage input
  const int first = blockIdx.x, step = gridDim.x, end = ntiles;

  if (warp == Tile::WARPS) {
    if (lane == 0) {
      int k = 0;
      BatchTile next = first < end ? tiles[first] : BatchTile{0, 0, 0, 0};
      for (int tile = first; tile < end; tile += step, k++) {
        const BatchTile tt = next;
        if (tile + step < end) next = tiles[tile + step];  // the next descriptor, read ahead
        const int b = k & 1;
        if (k >= 2 && !mbar_wait_bounded(&empty[b], ((k >> 1) - 1) & 1)) {
          atomicOr(err, ERR_TMA_TIMEOUT);
          break;
        }
        const int i0 = tt.i0, j0 = tt.j0;
        const CUtensorMap* m = maps + (long long)tt.slot * kBatchMaps;
        unsigned char* st = smem + b * Tile::STAGE_BYTES;
        mbar_arrive_expect_tx(&full[b], Tile::TX_BYTES);
        tma_load_3d(st, &m[3 * sel + 0], i0 - HX, j0 - HY, 2, &full[b]);
        tma_load_3d(st + Tile::OFF_U, &m[3 * sel + 1], i0 - HX, j0, 0, &full[b]);
        tma_load_3d(st + Tile::OFF_V, &m[3 * sel + 2], i0, j0 - HY, 1, &full[b]);
        if (Tile::LOAD_UN) tma_load_3d(st + Tile::OFF_N, &m[9], i0, j0, 0, &full[b]);
        if (Tile::LOAD_ACC) tma_load_3d(st + Tile::OFF_A, &m[10], i0, j0, 0, &full[b]);
        if (Tile::LOAD_COMP) tma_load_3d(st + Tile::OFF_C, &m[11], i0, j0, 0, &full[b]);
        bulk_copy_g2s(st + Tile::OFF_PRM, &insts[tt.slot], (uint32_t)sizeof(BatchWave<T>), &full[b]);
      }
      for (int kk = (k >= 2 ? k - 2 : 0); kk < k; kk++)
        if (!mbar_wait_bounded(&full[kk & 1], (kk >> 1) & 1)) atomicOr(err, ERR_TMA_TIMEOUT);
    }
    return;
  }

  uint32_t dphase = 0;  // parity of each stage's next deferred-pass barrier phase
  int k = 0;
  for (int tile = first; tile < end; tile += step, k++) {
    const int b = k & 1;
    if (!mbar_wait_bounded(&full[b], (k >> 1) & 1)) {
      if (lane == 0) atomicOr(err, ERR_TMA_TIMEOUT);
      break;
    }
    const unsigned char* st = smem + b * Tile::STAGE_BYTES;
    const BatchWave<T>& I = *reinterpret_cast<const BatchWave<T>*>(st + Tile::OFF_PRM);
    const BatchTile tt = tiles[tile];
    const int i0 = tt.i0, j0 = tt.j0;
    const T* in;
    T* wout;
    T c_acc, c_w;
    batch_stage_buffers(I, rk, in, wout, c_acc, c_w);
    wave_tile_compute<T, ORD, WK_CONST, STAGE, Tile>(I.prm, in, wout, c_acc, c_w, st, i0, j0, warp, lane, nullptr,
                                                     &dbar[b], &dphase, b, k);
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[b]);
  }
}

// Batched 2D advection: one CTA of 32 x 8 threads per 32 x 32 (instance, tile)
// pair, 4 rows per thread; the instance block is staged in shared memory once.
// Staging the tile's stage input with its halo in shared memory as well (a fill
// and a barrier per CTA) measured slower: batched FP32 6.67e10 against 7.27e10
// point-stage updates/s; the taps' reuse is served by L1.
template <typename T> struct alignas(16) BatchLine {
  LineParams<T> prm;  // geometry, taps, SAT factors, un/acc/comp pointers
  T* wa;
  T* wb;
  double dt;
  T c_acc[4], c_w[4];  // RK4 stage rk's coefficients at [rk - 1], computed on the host
};

constexpr int kLineTileX = 32, kLineTileY = 32, kLineThreadsY = 8;

template <typename T, int ORD, int STAGE>
__global__ void __launch_bounds__(kLineTileX * kLineThreadsY)
    adv_batch_stage_kernel(const BatchLine<T>* __restrict__ insts, const BatchTile* __restrict__ tiles, int rk) {
  __shared__ __align__(16) unsigned char blk[sizeof(BatchLine<T>)];
  const BatchTile tt = tiles[blockIdx.x];
  {
    const uint4* src = reinterpret_cast<const uint4*>(&insts[tt.slot]);
    uint4* dst = reinterpret_cast<uint4*>(blk);
    for (int k = threadIdx.y * kLineTileX + threadIdx.x; k < (int)(sizeof(BatchLine<T>) / 16);
         k += kLineTileX * kLineThreadsY)
      dst[k] = src[k];
  }
  __syncthreads();
  const BatchLine<T>& I = *reinterpret_cast<const BatchLine<T>*>(blk);
  const T* in = rk == 1 ? I.prm.un : (rk == 3 ? I.wb : I.wa);
  T* wout = (rk == 1 || rk == 3) ? I.wa : I.wb;
  const T c_acc = I.c_acc[rk - 1];
  const T c_w = I.c_w[rk - 1];
  const int i = tt.i0 + threadIdx.x;
  if (i >= I.prm.nx) return;
#pragma unroll
  for (int r = 0; r < kLineTileY / kLineThreadsY; r++) {
    const int j = tt.j0 + threadIdx.y + kLineThreadsY * r;
    if (j < I.prm.ny) line_point<T, ORD, LK_ADV2D, STAGE>(I.prm, in, wout, c_acc, c_w, i, j);
  }
}

}  // namespace sbp
