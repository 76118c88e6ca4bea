// wave_batch.cuh -- many independent wave / advection instances of uneven
// size, order and coefficients advanced together.
//
// Each (operator order, problem kind) group runs a persistent stage kernel whose
// grid walks a tile list of (instance, tile) pairs. The producer warp loads
// each tile's boxes with TMA from the instance's own tensor maps (kept in
// global memory) and bulk-copies the instance's parameter block (taps, SAT
// weights, pointers, time step) into the same shared-memory stage, so the
// compute warps read every per-instance constant from shared memory.
//
// Wave instances (rho = 1, K = c^2, one constant per instance): the tile
// arithmetic of the single-instance kernel (wave_tile_compute), or in FP64 its
// fixed-point stencils with converter warps (wave_tile_fixed). Advection
// instances (one component): taps from the stage input's box, the single-
// instance line kernel's operations and order. Each group's kernel shape comes
// from a small configuration table (below) that the autotuner chooses from.
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
  // FP64 fixed-point stages: stage rk's coefficients times each component's scale
  // (prm.fx_sig, and fx_sigp with K folded in), at [rk - 1]
  double fxa[4][3], fxw[4][3];
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

// A batched stage kernel's configuration: tile rows, compute warps, ring depth
// (tiles in flight) and resident CTAs per SM. Each (operator order, problem kind)
// group of a batch runs the configuration the autotuner picked from its table
// by timing the group's middle stage on the batch itself (sbp_batch_autotune);
// entry 0 is the default. Every entry fits the 227 KB of shared memory a CTA may
// use, and with 2 CTAs per SM the 228 KB of the SM (static_asserts below). More
// than 16 warps per SM leave 96 registers a thread, which the FP32 wave kernel
// with 16-row tiles and a 3-deep ring exceeds (it spilled): that entry has 8 warps.
// The FP64 fixed-point entry runs the single grid's shape (14 compute, 6 converter
// warps, 80 registers, a few spilled); with 7 compute warps it spills nothing but ran
// the 512-instance batch at 2.21e10 against 3.06e10 point-stage updates/s.
struct BatchCfg {
  int ty, warps, nst, ctas;
  int conv = 0;  // FP64 waves: converter warps of the fixed-point kernel (0: FP64 taps)
};
constexpr int kBatchCfgs = 4;
template <typename T> struct BatchCfgTable;
template <> struct BatchCfgTable<float> {
  static constexpr BatchCfg wave[kBatchCfgs] = {{32, 16, 2, 1}, {8, 8, 3, 2}, {16, 8, 2, 2}, {16, 8, 4, 1}};
  static constexpr BatchCfg adv[kBatchCfgs] = {{32, 8, 4, 1}, {16, 8, 4, 2}, {16, 4, 4, 2}, {32, 8, 2, 2}};
};
template <> struct BatchCfgTable<double> {
  static constexpr BatchCfg wave[kBatchCfgs] = {{16, 8, 2, 1}, {14, 14, 3, 1, 6}, {8, 8, 3, 1}, {8, 4, 2, 2}};
  static constexpr BatchCfg adv[kBatchCfgs] = {{16, 8, 4, 1}, {32, 8, 3, 1}, {16, 4, 3, 2}, {8, 4, 6, 2}};
};
template <typename T, int CFG> constexpr BatchCfg batch_wave_cfg() { return BatchCfgTable<T>::wave[CFG]; }
template <typename T, int CFG> constexpr BatchCfg batch_adv_cfg() { return BatchCfgTable<T>::adv[CFG]; }

template <typename T, int ORD, int STAGE, int CFG>
using BatchWaveTile = WaveTile<T, ORD, STAGE, batch_wave_cfg<T, CFG>().ty, (int)sizeof(BatchWave<T>), false,
                               batch_wave_cfg<T, CFG>().nst, batch_wave_cfg<T, CFG>().warps,
                               (batch_wave_cfg<T, CFG>().conv > 0), batch_wave_cfg<T, CFG>().conv>;

// A CTA takes every gridDim.x-th tile of the list, so neighbouring tiles of an
// instance run at the same time on neighbouring CTAs and share their halo rows in
// L2. Measured at 512 instances: contiguous ranges of the list per CTA ran at
// 1.39e10 (FP64) / 2.36e10 (FP32) point-stage updates/s against 1.72e10 / 3.22e10,
// and prefetching the next instance's tensor maps changed nothing.
template <typename T, int ORD, int STAGE, int CFG>
__global__ void __launch_bounds__(BatchWaveTile<T, ORD, STAGE, CFG>::THREADS, batch_wave_cfg<T, CFG>().ctas)
    wave_batch_stage_kernel(const BatchWave<T>* __restrict__ insts, const CUtensorMap* __restrict__ maps,
                            const BatchTile* __restrict__ tiles, int ntiles, int rk, int* err) {
  using Tile = BatchWaveTile<T, ORD, STAGE, CFG>;
  static_assert(batch_wave_cfg<T, CFG>().ctas * (Tile::SMEM + 1024) <= 228 * 1024, "CTAs per SM exceed shared memory");
  constexpr int HX = Tile::HX, HY = Tile::HY, NST = Tile::NST;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + Tile::OFF_BAR);
  uint64_t* empty = full + NST;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  uint64_t* dbar = reinterpret_cast<uint64_t*>(smem + Tile::OFF_DBAR);
  int2* origin = reinterpret_cast<int2*>(smem + Tile::OFF_BAR + 192);  // each stage's tile origin
  static_assert(NST <= 8, "tile origins: 64 bytes");
  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], Tile::WARPS);
      mbar_init(&dbar[s], Tile::WARPS);
    }
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
        const int b = k % NST;
        if (k >= NST && !mbar_wait_bounded(&empty[b], ((k / NST) - 1) & 1)) {
          atomicOr(err, ERR_TMA_TIMEOUT);
          break;
        }
        const int i0 = tt.i0, j0 = tt.j0;
        const CUtensorMap* m = maps + (long long)tt.slot * kBatchMaps;
        unsigned char* st = smem + b * Tile::STAGE_BYTES;
        origin[b] = make_int2(i0, j0);  // published by the arrive below
        mbar_arrive_expect_tx(&full[b], Tile::TX_BYTES);
        tma_load_3d(st, &m[3 * sel + 0], i0 - HX, j0 - HY, 2, &full[b]);
        tma_load_3d(st + Tile::OFF_U, &m[3 * sel + 1], i0 - HX, j0, 0, &full[b]);
        tma_load_3d(st + Tile::OFF_V, &m[3 * sel + 2], i0, j0 - HY, 1, &full[b]);
        if (Tile::LOAD_UN) tma_load_3d(st + Tile::OFF_N, &m[9], i0, j0, 0, &full[b]);
        if (Tile::LOAD_ACC) tma_load_3d(st + Tile::OFF_A, &m[10], i0, j0, 0, &full[b]);
        if (Tile::LOAD_COMP) tma_load_3d(st + Tile::OFF_C, &m[11], i0, j0, 0, &full[b]);
        bulk_copy_g2s(st + Tile::OFF_PRM, &insts[tt.slot], (uint32_t)sizeof(BatchWave<T>), &full[b]);
      }
      for (int kk = (k >= NST ? k - NST : 0); kk < k; kk++)
        if (!mbar_wait_bounded(&full[kk % NST], (kk / NST) & 1)) atomicOr(err, ERR_TMA_TIMEOUT);
    }
    return;
  }

  uint32_t dphase = 0;  // parity of each stage's next deferred-pass barrier phase
  int k = 0;
  for (int tile = first; tile < end; tile += step, k++) {
    const int b = k % NST;
    if (!mbar_wait_bounded(&full[b], (k / NST) & 1)) {
      if (lane == 0) atomicOr(err, ERR_TMA_TIMEOUT);
      break;
    }
    const unsigned char* st = smem + b * Tile::STAGE_BYTES;
    const BatchWave<T>& I = *reinterpret_cast<const BatchWave<T>*>(st + Tile::OFF_PRM);
    const int2 o0 = origin[b];
    const int i0 = o0.x, j0 = o0.y;
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

// The FP64 wave groups' fixed-point kernel (table entries with converter warps): the
// single grid's converter-warp stage (wave_fixed_kernel) over the batch's tile list. The
// producer loads each tile's boxes with its instance's tensor maps and bulk-copies the
// instance block into the stage, where the compute warps take the instance's parameters,
// its stage buffers and its scaled RK4 coefficients (fxa, fxw: K folded into p's).
template <typename Tile>
__device__ __forceinline__ void batch_fixed_produce(const BatchWave<double>* __restrict__ insts,
                                                    const CUtensorMap* __restrict__ maps,
                                                    const BatchTile* __restrict__ tiles, int ntiles, int rk,
                                                    unsigned char* smem, uint64_t* full, uint64_t* empty, int* tslot,
                                                    int2* origin, int* err) {
  constexpr int HX = Tile::HX, HY = Tile::HY, NST = Tile::NST;
  const int sel = rk == 1 ? 0 : (rk == 3 ? 2 : 1);  // which buffer is the stage input
  int k = 0;
  int tile = blockIdx.x;
  BatchTile next = tile < ntiles ? tiles[tile] : BatchTile{0, 0, 0, 0};
  for (;; k++) {
    const int b = k % NST;
    if (k >= NST && !mbar_wait_bounded(&empty[b], ((k / NST) - 1) & 1)) {
      atomicOr(err, ERR_TMA_TIMEOUT);
      break;
    }
    if (tile >= ntiles) {  // the end marker: a phase completed without bytes
      tslot[b] = -1;
      mbar_arrive(&full[b]);
      k++;
      break;
    }
    const BatchTile tt = next;
    tslot[b] = tile;
    origin[b] = make_int2(tt.i0, tt.j0);
    tile += gridDim.x;
    if (tile < ntiles) next = tiles[tile];  // the next descriptor, read ahead
    const CUtensorMap* m = maps + (long long)tt.slot * kBatchMaps;
    unsigned char* st = smem + b * Tile::STAGE_BYTES;
    mbar_arrive_expect_tx(&full[b], Tile::TX_BYTES);
    tma_load_3d(st, &m[3 * sel + 0], tt.i0 - HX, tt.j0 - HY, 2, &full[b]);
    tma_load_3d(st + Tile::OFF_U, &m[3 * sel + 1], tt.i0 - HX, tt.j0, 0, &full[b]);
    tma_load_3d(st + Tile::OFF_V, &m[3 * sel + 2], tt.i0, tt.j0 - HY, 1, &full[b]);
    if (Tile::LOAD_UN) tma_load_3d(st + Tile::OFF_N, &m[9], tt.i0, tt.j0, 0, &full[b]);
    if (Tile::LOAD_ACC) tma_load_3d(st + Tile::OFF_A, &m[10], tt.i0, tt.j0, 0, &full[b]);
    bulk_copy_g2s(st + Tile::OFF_PRM, &insts[tt.slot], (uint32_t)sizeof(BatchWave<double>), &full[b]);
  }
  // the CTA must not exit with copies in flight
  for (int kk = (k >= NST ? k - NST : 0); kk < k; kk++)
    if (!mbar_wait_bounded(&full[kk % NST], (kk / NST) & 1)) atomicOr(err, ERR_TMA_TIMEOUT);
}

template <int ORD, int STAGE, int CFG>
__global__ void __launch_bounds__(BatchWaveTile<double, ORD, STAGE, CFG>::THREADS, 1)
    wave_batch_fixed_kernel(const BatchWave<double>* __restrict__ insts, const CUtensorMap* __restrict__ maps,
                            const BatchTile* __restrict__ tiles, int ntiles, int rk, int* err) {
  using Tile = BatchWaveTile<double, ORD, STAGE, CFG>;
  constexpr int NST = Tile::NST, WARPS = Tile::WARPS, CONV = Tile::CONV;
  static_assert(Tile::FIX && CONV >= 1 && NST <= 4, "the converter-warp kernel; four tile origins");
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + Tile::OFF_BAR);
  uint64_t* empty = full + NST;
  uint64_t* dbar = reinterpret_cast<uint64_t*>(smem + Tile::OFF_DBAR);
  int* tslot = reinterpret_cast<int*>(smem + Tile::OFF_BAR + 192);
  int2* origin = reinterpret_cast<int2*>(smem + Tile::OFF_BAR + 224);
  uint64_t* fxa = reinterpret_cast<uint64_t*>(smem + Tile::OFF_FX);  // [8]: exponent maxima known
  uint64_t* conv = fxa + 8;                                          // [8]: stage converted
  int* wmax = reinterpret_cast<int*>(smem + Tile::OFF_FX + 128);     // [8][8][2]
  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], WARPS);
      mbar_init(&dbar[s], WARPS);
      mbar_init(&fxa[s], CONV);
      mbar_init(&conv[s], CONV);
    }
    fence_barrier_init();
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == WARPS + CONV) {
    if (lane == 0) batch_fixed_produce<Tile>(insts, maps, tiles, ntiles, rk, smem, full, empty, tslot, origin, err);
    return;
  }
  if (warp >= WARPS) {  // ---- converters
    const int t = threadIdx.x - 32 * WARPS;
    for (int k = 0;; k++) {
      const int b = k % NST;
      if (!mbar_wait_bounded(&full[b], (k / NST) & 1)) {
        if (lane == 0) atomicOr(err, ERR_TMA_TIMEOUT);
        break;
      }
      const int tile = tslot[b];
      if (tile >= 0 &&
          !fx_convert_stage<Tile>(smem + b * Tile::STAGE_BYTES, &fxa[b], wmax + 16 * b, (k / NST) & 1, 0, t)) {
        if (lane == 0) atomicOr(err, ERR_TMA_TIMEOUT);
        break;
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&conv[b]);  // converted, or the end marker passed on
      if (tile < 0) break;
    }
    return;
  }
  // ---- compute warps
  uint32_t dphase = 0;  // parity of each stage's next deferred-pass barrier phase
  for (int k = 0;; k++) {
    const int b = k % NST;
    if (!mbar_wait_bounded(&conv[b], (k / NST) & 1)) {
      if (lane == 0) atomicOr(err, ERR_TMA_TIMEOUT);
      break;
    }
    if (tslot[b] < 0) break;
    const unsigned char* st = smem + b * Tile::STAGE_BYTES;
    const BatchWave<double>& I = *reinterpret_cast<const BatchWave<double>*>(st + Tile::OFF_PRM);
    const int2 o0 = origin[b];
    const double* in;
    double* wout;
    double c_acc, c_w;
    batch_stage_buffers(I, rk, in, wout, c_acc, c_w);
    int ep, euv;
    bool bad;
    fx_tile_emax<CONV>(wmax + 16 * b, ep, euv, bad);
    const FxGeom g{I.prm.nx, I.prm.ny, 0, 0, 0, 0, I.prm.pitch, I.prm.plane, 0};
    wave_tile_fixed<ORD, STAGE, Tile, WK_CONST>(I.prm, g, in, wout, c_acc, c_w, I.fxa[rk - 1], I.fxw[rk - 1], st, o0.x,
                                                o0.y, warp, lane, ep, euv, bad, &dbar[b], &dphase, b, k);
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[b]);
  }
}

// Per-instance block of a batched advection instance (16-byte multiple, bulk-copied
// into shared memory beside each tile).
template <typename T> struct alignas(16) BatchLine {
  LineParams<T> prm;  // geometry, taps (velocities folded in), SAT factors, un/acc/comp pointers
  T* wa;
  T* wb;
  double dt;
  T c_acc[4], c_w[4];  // RK4 stage rk's coefficients at [rk - 1], computed on the host
};

// Tensor maps of one batched advection instance (one component), in global memory:
// [s] = stage input s (0: u^n, 1: wa, 2: wb) with the tile box and its halo;
// [3], [4], [5] = u^n, acc, comp point boxes.
constexpr int kAdvMaps = 6;

// The shared-memory stage of the batched advection kernel: the stage input's
// box (tile + R halo lines each side; x halo rounded up to 16 bytes), the u^n,
// acc and comp point boxes the stage reads, and the instance block.
template <typename T, int ORD, int STAGE, int CFG>
struct AdvTile {
  static constexpr BatchCfg C = batch_adv_cfg<T, CFG>();
  static constexpr int TY = C.ty, WARPS = C.warps, NST = C.nst, THREADS = 32 * (WARPS + 1);
  static constexpr int R = (OpShape<ORD>::W - 1) / 2;
  static constexpr int HXA = 16 / sizeof(T);
  static constexpr int HX = ((R + HXA - 1) / HXA) * HXA, HY = R;
  static constexpr int PW = kWaveTX + 2 * HX, PH = TY + 2 * HY;
  static constexpr bool COMP = sizeof(T) == 4;  // FP32: compensated RK4 update
  static constexpr bool LOAD_UN = (STAGE == ST_MID) || (STAGE == ST_LAST && COMP);
  static constexpr bool LOAD_ACC = (STAGE == ST_MID) || (STAGE == ST_LAST);
  static constexpr bool LOAD_COMP = (STAGE == ST_LAST && COMP);
  static constexpr int align128(int b) { return (b + 127) / 128 * 128; }
  static constexpr int BYTES_P = PH * PW * (int)sizeof(T);
  static constexpr int BYTES_PT = TY * kWaveTX * (int)sizeof(T);
  static constexpr int OFF_N = align128(BYTES_P);
  static constexpr int OFF_A = OFF_N + (LOAD_UN ? BYTES_PT : 0);
  static constexpr int OFF_C = OFF_A + (LOAD_ACC ? BYTES_PT : 0);
  static constexpr int OFF_PRM = align128(OFF_C + (LOAD_COMP ? BYTES_PT : 0));
  // the RHS and centre value of the tile's x-face points, kept for the deferred SAT pass ([side][row][2])
  static constexpr int OFF_DEF = OFF_PRM + align128((int)sizeof(BatchLine<T>));
  static constexpr int STAGE_BYTES = OFF_DEF + align128(2 * TY * 2 * (int)sizeof(T));
  // full[8] (+0), empty[8] (+64), deferred-pass barriers[8] (+128), tile origins int2[8] (+192)
  static constexpr int OFF_BAR = NST * STAGE_BYTES;
  static constexpr int SMEM = OFF_BAR + 256;
  static constexpr uint32_t TX_BYTES = BYTES_P + (LOAD_UN ? BYTES_PT : 0) + (LOAD_ACC ? BYTES_PT : 0) +
                                       (LOAD_COMP ? BYTES_PT : 0) + (int)sizeof(BatchLine<T>);
  static_assert(TY % WARPS == 0, "tile rows must split evenly over the compute warps");
  static_assert(NST >= 2 && NST <= 8, "ring depth");
  static_assert(SMEM <= 227 * 1024, "advection tile pipeline exceeds shared memory");
  static_assert(C.ctas * (SMEM + 1024) <= 228 * 1024, "CTAs per SM exceed shared memory");
};



// Batched 2D advection u_t = -(a u_x + b u_y) (code/demo/advection/advection_rhs.h:155-393,
// 460-528), persistent like the wave kernel: the producer warp loads each (instance,
// tile) pair's boxes with the instance's tensor maps, bulk-copies its parameter block
// beside them and writes the tile's origin into the stage's slot, in a ring of NST
// stages; each compute warp takes TY / WARPS rows of 64 points (two per lane). Taps
// read the stage input's box -- closure rows too, where their stencil lies inside it
// (else global memory) -- in the single-instance line kernel's order, so both give
// the same bits. The SAT is FP64: inline at y-face points (whole warp rows), and for
// the x-face points, which hold one lane of a row each, in a deferred pass of one warp
// over the tile's two x faces (one FP64 sequence per 32 face points instead of one
// per row). A CTA takes every gridDim.x-th tile.
template <typename T, int ORD, int STAGE, int CFG>
__global__ void __launch_bounds__(AdvTile<T, ORD, STAGE, CFG>::THREADS, batch_adv_cfg<T, CFG>().ctas)
    adv_batch_stage_kernel(const BatchLine<T>* __restrict__ insts, const CUtensorMap* __restrict__ maps,
                           const BatchTile* __restrict__ tiles, int ntiles, int rk, int* err) {
  using Tile = AdvTile<T, ORD, STAGE, CFG>;
  constexpr int HX = Tile::HX, HY = Tile::HY, NST = Tile::NST, WARPS = Tile::WARPS, PW = Tile::PW, TY = Tile::TY;
  constexpr int W = OpShape<ORD>::W, CS = OpShape<ORD>::CS, CW = OpShape<ORD>::CW, R = Tile::R;
  constexpr int ROWS = TY / WARPS;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + Tile::OFF_BAR);
  uint64_t* empty = full + 8;
  uint64_t* dbar = full + 16;
  int2* origin = reinterpret_cast<int2*>(smem + Tile::OFF_BAR + 192);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], WARPS);
      mbar_init(&dbar[s], WARPS);
    }
    fence_barrier_init();
  }
  __syncthreads();
  const int sel = rk == 1 ? 0 : (rk == 3 ? 2 : 1);  // which buffer is the stage input
  const int first = blockIdx.x, step = gridDim.x, end = ntiles;

  if (warp == WARPS) {  // producer
    if (lane == 0) {
      int k = 0;
      BatchTile next = first < end ? tiles[first] : BatchTile{0, 0, 0, 0};
      for (int tile = first; tile < end; tile += step, k++) {
        const BatchTile tt = next;
        if (tile + step < end) next = tiles[tile + step];  // the next descriptor, read ahead
        const int b = k % NST;
        if (k >= NST && !mbar_wait_bounded(&empty[b], ((k / NST) - 1) & 1)) {
          atomicOr(err, ERR_TMA_TIMEOUT);
          break;
        }
        const CUtensorMap* m = maps + (long long)tt.slot * kAdvMaps;
        unsigned char* st = smem + b * Tile::STAGE_BYTES;
        origin[b] = make_int2(tt.i0, tt.j0);  // published by the arrive below
        mbar_arrive_expect_tx(&full[b], Tile::TX_BYTES);
        tma_load_3d(st, &m[sel], tt.i0 - HX, tt.j0 - HY, 0, &full[b]);
        if (Tile::LOAD_UN) tma_load_3d(st + Tile::OFF_N, &m[3], tt.i0, tt.j0, 0, &full[b]);
        if (Tile::LOAD_ACC) tma_load_3d(st + Tile::OFF_A, &m[4], tt.i0, tt.j0, 0, &full[b]);
        if (Tile::LOAD_COMP) tma_load_3d(st + Tile::OFF_C, &m[5], tt.i0, tt.j0, 0, &full[b]);
        bulk_copy_g2s(st + Tile::OFF_PRM, &insts[tt.slot], (uint32_t)sizeof(BatchLine<T>), &full[b]);
      }
      for (int kk = (k >= NST ? k - NST : 0); kk < k; kk++)
        if (!mbar_wait_bounded(&full[kk % NST], (kk / NST) & 1)) atomicOr(err, ERR_TMA_TIMEOUT);
    }
    return;
  }

  uint32_t dphase = 0;  // parity of each stage's next deferred-pass barrier phase
  int k = 0;
  for (int tile = first; tile < end; tile += step, k++) {
    const int b = k % NST;
    if (!mbar_wait_bounded(&full[b], (k / NST) & 1)) {
      if (lane == 0) atomicOr(err, ERR_TMA_TIMEOUT);
      break;
    }
    const unsigned char* st = smem + b * Tile::STAGE_BYTES;
    const BatchLine<T>& I = *reinterpret_cast<const BatchLine<T>*>(st + Tile::OFF_PRM);
    const LineParams<T>& prm = I.prm;
    const T* sP = reinterpret_cast<const T*>(st);
    const T* sN = reinterpret_cast<const T*>(st + Tile::OFF_N);
    const T* sA = reinterpret_cast<const T*>(st + Tile::OFF_A);
    const T* sC = reinterpret_cast<const T*>(st + Tile::OFF_C);
    T* sD = reinterpret_cast<T*>(const_cast<unsigned char*>(st) + Tile::OFF_DEF);
    const int2 o0 = origin[b];
    const int i0 = o0.x, j0 = o0.y;
    const T* in = rk == 1 ? prm.un : (rk == 3 ? I.wb : I.wa);
    T* wout = (rk == 1 || rk == 3) ? I.wa : I.wb;
    const T c_acc = I.c_acc[rk - 1], c_w = I.c_w[rk - 1];
    const int nx = prm.nx, ny = prm.ny;
    const long long pitch = prm.pitch;
    // closure stencils inside the box (columns i0 - HX .. i0 + 64 + HX - 1, rows j0 - HY ..
    // j0 + TY + HY - 1): the first CW points of a line when the tile starts it, the last CW
    // when they neither start before nor end after the box
    static_assert(CW <= kWaveTX && CW <= TY + HY, "a tile that starts a line holds its closure stencil");
    const bool xl_in = i0 == 0, xr_in = nx - CW >= i0 - HX && nx <= i0 + kWaveTX + HX;
    const bool yl_in = j0 == 0, yr_in = ny - CW >= j0 - HY && ny <= j0 + TY + HY;
    const bool xfaces = prm.bc && (i0 == 0 || i0 + kWaveTX >= nx);  // the tile holds column 0 or nx - 1
    // the RK4 stage update of point (i, j), (x, y) in the tile
    auto store = [&](int i, int j, int x, int y, T kk, T cen) {
      const long long o = (long long)j * pitch + i;
      const int p = y * kWaveTX + x;  // the point in a point box
      if constexpr (STAGE == ST_FIRST) {
        prm.acc[o] = Tile::COMP ? c_acc * kk : fma(c_acc, kk, cen);
        wout[o] = fma(c_w, kk, cen);
      } else if constexpr (STAGE == ST_MID) {
        prm.acc[o] = fma(c_acc, kk, sA[p]);
        wout[o] = fma(c_w, kk, sN[p]);
      } else {
        const T d = fma(c_acc, kk, sA[p]);
        if constexpr (Tile::COMP) {  // Kahan: u^n + d with the carried error
          const T u0 = sN[p], e = sC[p];
          const T yv = d - e;
          const T tv = u0 + yv;
          prm.comp[o] = (tv - u0) - yv;
          prm.un[o] = tv;
        } else {
          prm.un[o] = d;
        }
      }
    };
#pragma unroll
    for (int rr = 0; rr < ROWS; rr++) {
      const int y = warp * ROWS + rr, j = j0 + y;
      if (j >= ny) break;
#pragma unroll
      for (int cc = 0; cc < kWaveTX / 32; cc++) {
        const int x = lane + 32 * cc, i = i0 + x;
        if (i >= nx) continue;
        const T* c = sP + (y + HY) * PW + (x + HX);  // the point in the stage input's box
        T kx, ky;
        if (i >= CS && i < nx - CS) {
          kx = prm.dx.taps[0] * c[-R];
#pragma unroll
          for (int s = 1; s < W; s++)
            if (s != R) kx = fma(prm.dx.taps[s], c[s - R], kx);
        } else if (i < CS ? xl_in : xr_in) {
          kx = closure_line_smem<T, ORD>(c - i, 1, nx, i, prm.dx.cls);  // c - i: the line's point 0
        } else {
          kx = closure_line_global<T, ORD>(in + (long long)j * pitch, 1, nx, i, prm.dx.cls);
        }
        if (j >= CS && j < ny - CS) {
          ky = prm.dy.taps[0] * c[-R * PW];
#pragma unroll
          for (int s = 1; s < W; s++)
            if (s != R) ky = fma(prm.dy.taps[s], c[(s - R) * PW], ky);
        } else if (j < CS ? yl_in : yr_in) {
          ky = closure_line_smem<T, ORD>(c - j * PW, PW, ny, j, prm.dy.cls);
        } else {
          ky = closure_line_global<T, ORD>(in + i, pitch, ny, j, prm.dy.cls);
        }
        const T cen = *c;
        if (xfaces && (i == 0 || i == nx - 1)) {  // x-face point: its SAT in the deferred pass
          T* d = sD + ((i == 0 ? 0 : TY) + y) * 2;
          d[0] = kx + ky;
          d[1] = cen;
          continue;
        }
        store(i, j, x, y, adv2d_sat<T>(prm, i, j, kx + ky, cen), cen);
      }
    }
    if (xfaces) {
      __syncwarp();
      if (lane == 0) mbar_arrive(&dbar[b]);  // this warp's deferred entries are in shared memory
      const uint32_t par = (dphase >> b) & 1u;
      dphase ^= 1u << b;
      if (warp == k % WARPS) {
        if (!mbar_wait_bounded(&dbar[b], par)) {
          if (lane == 0) atomicOr(err, ERR_TMA_TIMEOUT);
        } else {
          for (int e = lane; e < 2 * TY; e += 32) {
            const int side = e / TY, y = e - side * TY, j = j0 + y;
            const int i = side == 0 ? 0 : nx - 1;
            if (j >= ny || i < i0 || i >= i0 + kWaveTX) continue;
            const T* d = sD + (side * TY + y) * 2;
            store(i, j, i - i0, y, adv2d_sat<T>(prm, i, j, d[0], d[1]), d[1]);
          }
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[b]);
  }
}

}  // namespace sbp
