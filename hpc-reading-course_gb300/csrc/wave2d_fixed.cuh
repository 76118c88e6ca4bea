// wave2d_fixed.cuh -- the FP64 constant-coefficient wave stage (rho = K = 1)
// with its interior stencils in exact integer arithmetic.
//
// GB300 issues FP64 FMAs at about 1/64 of its FP32 rate, and the FP64 tap
// chains of wave_tile_compute (4 derivatives x 4 taps at order 4, plus the
// stage update) keep that pipe busy long before HBM is. The interior stencils
// of the central SBP operators have rational weights with a small common
// denominator (code/include/sbpops/D1_central.h:245,254,266):
//     order 2: (1/2)  (v1 - v-1)
//     order 4: (1/12) (8 (v1 - v-1) - (v2 - v-2))
//     order 6: (1/60) (45 (v1 - v-1) - 9 (v2 - v-2) + (v3 - v-3))
// so den * sum is an integer combination of the point values. Each tile's
// stencil boxes are converted once, in place, to 64-bit integers in units of
// 2^(Emax - 1075), where Emax is the largest biased exponent among the box
// values of the group (p; u and v together): a double +-M 2^(E-1075) with its
// 53-bit mantissa M becomes +-round(M / 2^(Emax - E)), |V| < 2^53. The sums
// are then exact in int64 (|S| < 110 * 2^54 < 2^61 at order 6, and the sum of
// the u and v terms as well), and one conversion back to a double, rounded to
// nearest, carries the only rounding of the stencil: the result is as accurate
// as the reference's FP64 evaluation (the conversion to fixed point rounds each
// value to 2^-53 of the box's largest magnitude, the FP64 sum rounds each
// partial sum to 2^-53 of its own). The integer work runs on the INT pipe; the
// FP64 pipe is left with the RK4 stage update, 1-2 FMAs per component, into
// which the scale sigma = -hi/den is folded (fx_ca, fx_cw).
//
// Closure rows (boundary strips) keep the FP64 taps read from global memory
// and are brought to the same units by 1/sigma; SAT terms are applied in FP64
// in true units as in wave_tile_compute. A box holding a non-finite value gives
// NaN for every point of its tile.
#pragma once

#include "sbp_device.cuh"

namespace sbp {

template <int ORD> struct FixDen;
template <> struct FixDen<2> { static constexpr int value = 2; };
template <> struct FixDen<4> { static constexpr int value = 12; };
template <> struct FixDen<6> { static constexpr int value = 60; };

// v (given as its two 32-bit words) as a signed integer in units of
// 2^(emax - 1075), truncated towards zero; emax >= the exponent of v. Zero and
// subnormal values give 0, as does any shift of 64 or more.
__device__ __forceinline__ long long fx_from(unsigned lo, unsigned hi, int emax) {
  const unsigned e = (hi >> 20) & 0x7FFu;
  const unsigned mh = (hi & 0x000FFFFFu) | 0x00100000u;  // the 53-bit mantissa is mh:lo
  const unsigned sh = e == 0 ? 64u : (unsigned)emax - e;
  const unsigned rlo = sh < 32 ? __funnelshift_rc(lo, mh, sh) : __funnelshift_rc(mh, 0u, sh - 32u);
  const unsigned rhi = __funnelshift_rc(mh, 0u, sh);
  const long long r = (long long)(((unsigned long long)rhi << 32) | rlo);
  const long long sg = (long long)((int)hi >> 31);  // 0 or -1
  return (r ^ sg) - sg;
}

// s * 2^(eb - 11 - 1075) as a double, truncated towards zero (eb = emax + 11 of
// the box; the tile guard keeps emax in [64, 2030], so the exponent stays normal).
__device__ __forceinline__ double fx_to(long long s, int eb) {
  const long long sg = s >> 63;
  const unsigned long long a = (unsigned long long)((s ^ sg) - sg);
  const int lz = __clzll((long long)a);                        // >= 2: |s| < 2^62
  const unsigned long long n = a << (lz & 63);                  // leading one at bit 63
  const unsigned mh = (unsigned)(n >> 43);                      // leading one + 20 fraction bits
  const unsigned ml = (unsigned)(n >> 11);                      // the other 32 fraction bits
  const unsigned hw = (((unsigned)(eb - lz - 1)) << 20) + mh;   // the leading one adds the last 1 to the exponent
  const double r = __hiloint2double((int)(hw | ((unsigned)sg & 0x80000000u)), (int)ml);
  return a == 0 ? 0.0 : r;
}

// den * (interior stencil sum) at the point c of an int64 line with stride st.
template <int ORD>
__device__ __forceinline__ long long fx_stencil(const long long* c, int st) {
  if constexpr (ORD == 2) {
    return c[st] - c[-st];
  } else if constexpr (ORD == 4) {
    return 8 * (c[st] - c[-st]) - (c[2 * st] - c[-2 * st]);
  } else {
    return 45 * (c[st] - c[-st]) - 9 * (c[2 * st] - c[-2 * st]) + (c[3 * st] - c[-3 * st]);
  }
}

// Converts the p, u and v boxes of one ring stage to int64 in place (all
// consumer threads). Each thread keeps its elements in registers between the
// two barriers, both with bounded waits: the exponent maxima are known (fxa),
// the boxes are converted (fxb). Returns false if a wait ran out. emax[0..1]
// are the p and u/v maxima; a box whose maximum is below 64 (values under
// 2^-959) converts to zeros, and one at 2031 or more (values from 2^1008, Inf,
// NaN) marks the tile bad: its points get NaN.
template <typename Tile>
__device__ __forceinline__ bool fx_convert_tile(unsigned char* st, uint64_t* fxa, uint64_t* fxb, int* fxmax,
                                                uint32_t parity, unsigned long long wait_ns, int tid, int (&emax)[2],
                                                bool& bad) {
  constexpr int NT = 32 * Tile::WARPS;
  constexpr int NP = Tile::PH * Tile::PW, NU = Tile::TY * Tile::PW, NV = Tile::PH * kWaveTX;
  constexpr int CP = (NP + NT - 1) / NT, CU = (NU + NT - 1) / NT, CV = (NV + NT - 1) / NT;
  uint2* wP = reinterpret_cast<uint2*>(st);
  uint2* wU = reinterpret_cast<uint2*>(st + Tile::OFF_U);
  uint2* wV = reinterpret_cast<uint2*>(st + Tile::OFF_V);
  const int lane = tid & 31;
  uint2 rp[CP], ru[CU], rv[CV];
  unsigned mp = 0, muv = 0;
#pragma unroll
  for (int c = 0; c < CP; c++) {
    const int e = tid + c * NT;
    rp[c] = (c < NP / NT || e < NP) ? wP[e] : make_uint2(0u, 0u);
    mp = max(mp, rp[c].y & 0x7FF00000u);
  }
#pragma unroll
  for (int c = 0; c < CU; c++) {
    const int e = tid + c * NT;
    ru[c] = (c < NU / NT || e < NU) ? wU[e] : make_uint2(0u, 0u);
    muv = max(muv, ru[c].y & 0x7FF00000u);
  }
#pragma unroll
  for (int c = 0; c < CV; c++) {
    const int e = tid + c * NT;
    rv[c] = (c < NV / NT || e < NV) ? wV[e] : make_uint2(0u, 0u);
    muv = max(muv, rv[c].y & 0x7FF00000u);
  }
  mp = __reduce_max_sync(0xffffffffu, mp);
  muv = __reduce_max_sync(0xffffffffu, muv);
  if (lane == 0) {
    atomicMax(&fxmax[0], (int)(mp >> 20));
    atomicMax(&fxmax[1], (int)(muv >> 20));
  }
  __syncwarp();
  if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(fxa)) : "memory");
  if (!mbar_wait_bounded(fxa, parity, wait_ns)) return false;
  int ep = fxmax[0], euv = fxmax[1];
  bad = ep >= 2031 || euv >= 2031;
  if (ep < 64) ep = 2111;  // every value converts to 0
  if (euv < 64) euv = 2111;
  long long* iP = reinterpret_cast<long long*>(wP);
  long long* iU = reinterpret_cast<long long*>(wU);
  long long* iV = reinterpret_cast<long long*>(wV);
#pragma unroll
  for (int c = 0; c < CP; c++) {
    const int e = tid + c * NT;
    if (c < NP / NT || e < NP) iP[e] = fx_from(rp[c].x, rp[c].y, ep);
  }
#pragma unroll
  for (int c = 0; c < CU; c++) {
    const int e = tid + c * NT;
    if (c < NU / NT || e < NU) iU[e] = fx_from(ru[c].x, ru[c].y, euv);
  }
#pragma unroll
  for (int c = 0; c < CV; c++) {
    const int e = tid + c * NT;
    if (c < NV / NT || e < NV) iV[e] = fx_from(rv[c].x, rv[c].y, euv);
  }
  __syncwarp();
  if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(fxb)) : "memory");
  if (!mbar_wait_bounded(fxb, parity, wait_ns)) return false;
  // every consumer has read the maxima: clear them for the stage's next tile (its
  // atomics come after this warp's arrivals on the next tile's barriers)
  if (tid == 0) fxmax[0] = fxmax[1] = 0;
  emax[0] = ep;
  emax[1] = euv;
  return true;
}

// Where a tile's points live: the interior extent of the arrays holding them
// (the grid, or one subdomain of a decomposed grid), the global index of their
// first interior point, that point's array column and row (ghost lines before
// it), the row pitch, the component plane and the arrays' offset in the stage's
// buffers. The single grid: offsets zero, the arrays the whole buffers.
struct FxGeom {
  int nx, ny;
  int xoff, yoff;
  int col0, row0;
  long long pitch, plane, base;
};

// A subdomain of a decomposed grid: its interior points, the global index of its
// first interior point, and its arrays (row pitch, component plane, offset in the
// stage's buffers). Its first interior point sits at array column Tile::HX (the x
// ghost width, rounded up so every TMA x coordinate is 16-byte aligned) and row
// Tile::HY; the R ghost lines next to the interior hold the neighbours' values.
struct FxSub {
  int nx, ny, xoff, yoff;
  long long pitch, plane, base;
  int nbr[4];  // the neighbouring subdomain to the west, east, south, north, or -1
};
struct FxTile {
  int sub, i0, j0, pad;  // subdomain and tile origin in its interior indices
};

// A decomposed grid's tile as the producer hands it to the compute warps through
// shared memory (its geometry and origin), so they need no global loads per tile.
// A neighbour's arrays as a stage writes into its ghost lines: offset, row pitch,
// component plane and its interior extent across the shared edge (nx for a
// west/east neighbour, ny for a south/north one); n < 0 for none.
struct FxNbr {
  long long base, pitch, plane;
  int n, pad;
};
struct FxTileInfo {
  FxGeom g;
  int i0, j0;
  FxNbr nb[4];  // west, east, south, north
};
// Each tile's block in device memory (built by the host) and in a ring stage's slot:
// 192 bytes, a multiple of 16 for the bulk copy.
constexpr int kFxTileInfoBytes = 192;
static_assert(sizeof(FxTileInfo) <= kFxTileInfoBytes, "tile information slot");

// Decomposed grids: the halo exchange fused into the stages that produce the next
// stage input (the reference's VecScatter ghost update,
// code/src/scatter/scatter_ctx.cpp:149-211). Once a tile is done, each of its points
// within R of an edge shared with a neighbour copies its new value (w, or u^n in the
// last stage) into the neighbour's ghost line that mirrors it, so the next stage finds
// every ghost it reads without a separate exchange. Run by the 32 lanes of the
// exchange warp after the compute warps released the tile. The copies are enumerated
// side by side (each side's strip of the tile, component-major), and each lane issues
// U loads before its U stores, so one batch costs about two memory latencies.
template <typename Tile, int STAGE>
__device__ __forceinline__ void fx_exchange_tile(const WaveParams<double>& prm, const FxTileInfo& T, int lane) {
  constexpr int R = Tile::R, TY = Tile::TY, COL0 = Tile::HX, U = 4;
  const FxGeom& g = T.g;
  const int ie = min(T.i0 + kWaveTX, g.nx), je = min(T.j0 + TY, g.ny);
  // each side's strip of the tile, in the subdomain's interior indices: columns
  // [T.i0, iw) west, [ia, ie) east, rows [T.j0, js) south, [ja, je) north; the
  // strips of the sides without a neighbour are empty
  const int iw = min(ie, R), ia = max(T.i0, g.nx - R), js = min(je, R), ja = max(T.j0, g.ny - R);
  const int rows = je - T.j0, cols = ie - T.i0;
  const int c0 = T.nb[0].n >= 0 && iw > T.i0 ? 3 * (iw - T.i0) * rows : 0;
  const int c1 = T.nb[1].n >= 0 && ie > ia ? 3 * (ie - ia) * rows : 0;
  const int c2 = T.nb[2].n >= 0 && js > T.j0 ? 3 * cols * (js - T.j0) : 0;
  const int c3 = T.nb[3].n >= 0 && je > ja ? 3 * cols * (je - ja) : 0;
  const int total = c0 + c1 + c2 + c3;
  if (total == 0) return;
  double* obuf = STAGE == ST_LAST ? prm.un : prm.wout;
  for (int e0 = 0; e0 < total; e0 += 32 * U) {
    double v[U];
    long long dst[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      int e = e0 + lane + 32 * u;
      dst[u] = -1;
      if (e >= total) continue;
      int s, x0, w, y0, h;  // the side and its strip
      if (e < c0) {
        s = 0, x0 = T.i0, w = iw - T.i0, y0 = T.j0, h = rows;
      } else if ((e -= c0) < c1) {
        s = 1, x0 = ia, w = ie - ia, y0 = T.j0, h = rows;
      } else if ((e -= c1) < c2) {
        s = 2, x0 = T.i0, w = cols, y0 = T.j0, h = js - T.j0;
      } else {
        e -= c2;
        s = 3, x0 = T.i0, w = cols, y0 = ja, h = je - ja;
      }
      const int wh = w * h, c = e / wh, r = e - c * wh, j = y0 + r / w, i = x0 + r % w;
      v[u] = obuf[g.base + c * g.plane + (long long)(j + g.row0) * g.pitch + (i + g.col0)];
      const FxNbr& N = T.nb[s];
      const long long row = s == 0 || s == 1 ? j + g.row0 : (s == 2 ? N.n + j + g.row0 : j - g.ny + g.row0);
      const int col = s == 0 ? N.n + i + COL0 : (s == 1 ? i - g.nx + COL0 : i + COL0);
      dst[u] = N.base + c * N.plane + row * N.pitch + col;
    }
#pragma unroll
    for (int u = 0; u < U; u++)
      if (dst[u] >= 0) obuf[dst[u]] = v[u];
  }
}

// The threads of a fixed-point stage kernel: compute, converter and producer warps,
// and on a decomposed grid the exchange warp.
template <typename Tile, bool DEC>
constexpr int fx_kernel_threads() {
  return Tile::THREADS + (DEC ? 32 : 0);
}

// The exchange queue of a decomposed grid: the producer hands each released tile's
// geometry block to the exchange warp through the shared-memory slots after the NST
// ring stages' ones (Tile::OFF_TINFO), with a full/empty barrier pair per slot.
template <typename Tile>
struct FxExchangeQueue {
  static constexpr int SLOTS = 8 - Tile::NST;
  static_assert(SLOTS >= 2, "the tile geometry area leaves the exchange queue too few slots");
  unsigned char* slot0;
  uint64_t* full;
  uint64_t* empty;
  __device__ FxExchangeQueue(unsigned char* smem)
      : slot0(smem + Tile::OFF_TINFO + kFxTileInfoBytes * Tile::NST),
        full(reinterpret_cast<uint64_t*>(smem + Tile::OFF_XBAR)),
        empty(reinterpret_cast<uint64_t*>(smem + Tile::OFF_XBAR + 64)) {}
  __device__ FxTileInfo* slot(int s) const { return reinterpret_cast<FxTileInfo*>(slot0 + kFxTileInfoBytes * s); }
  // Push number q (all 32 lanes of the producer warp): the geometry block `from`, or
  // the end marker (i0 = -1) for nullptr. False if the wait for a free slot ran out.
  __device__ bool push(int q, const unsigned char* from, int lane, const WaveParams<double>& prm) const {
    const int s = q % SLOTS;
    if (q >= SLOTS && !mbar_wait_bounded(&empty[s], ((q / SLOTS) - 1) & 1, prm.wait_ns)) {
      if (lane == 0) atomicOr(prm.err, ERR_TMA_TIMEOUT);
      return false;
    }
    int4* to = reinterpret_cast<int4*>(slot(s));
    if (from) {
      if (lane < kFxTileInfoBytes / 16) to[lane] = reinterpret_cast<const int4*>(from)[lane];
    } else if (lane == 0) {
      slot(s)->i0 = -1;
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&full[s]);
    return true;
  }
};

// The exchange warp of a decomposed grid: takes the released tiles' geometry blocks
// from the exchange queue and runs their fused exchange, until the end marker. The
// compute warps' stores reach it through the ring stage's `empty` barrier and the
// queue's `full` barrier. Every wait is bounded.
template <typename Tile, int STAGE>
__device__ __forceinline__ void decomp_exchange(const WaveParams<double>& prm, const FxExchangeQueue<Tile>& xq,
                                                int lane) {
  constexpr int SLOTS = FxExchangeQueue<Tile>::SLOTS;
  for (int q = 0;; q++) {
    const int s = q % SLOTS;
    if (!mbar_wait_bounded(&xq.full[s], (q / SLOTS) & 1, prm.wait_ns)) {
      if (lane == 0) atomicOr(prm.err, ERR_TMA_TIMEOUT);
      return;
    }
    const FxTileInfo& T = *xq.slot(s);
    if (T.i0 < 0) return;
    fx_exchange_tile<Tile, STAGE>(prm, T, lane);
    __syncwarp();
    if (lane == 0) mbar_arrive(&xq.empty[s]);
  }
}

// The producer warp of a decomposed grid: lane 0 takes the tiles (dynamic queue or
// fixed stride) and issues each stage's loads -- TMA boxes with the maps of the tile's
// subdomain, and the tile's geometry block by a bulk copy on the stage's barrier --
// reading the next tile's descriptor one tile ahead. In the stages that produce the
// next stage input, each tile the compute warps release goes to the exchange queue
// (its geometry block copied by the 32 lanes) before its ring stage is refilled; the
// tiles still held at the end follow after their release, then the end marker.
// Every wait is bounded.
template <typename Tile, int STAGE>
__device__ __forceinline__ void decomp_produce(const WaveParams<double>& prm, unsigned char* smem, uint64_t* full,
                                               uint64_t* empty, int* tslot, const FxExchangeQueue<Tile>& xq,
                                               int lane) {
  constexpr int HY = Tile::HY, HX = Tile::HX, NST = Tile::NST;
  constexpr bool EXCH = STAGE == ST_FIRST || STAGE == ST_MID || STAGE == ST_LAST;
  const int ntiles = prm.dntiles;
  const bool dyn = prm.sched != nullptr;
  const unsigned char* tinfo = smem + Tile::OFF_TINFO;
  int k = 0, issued = 0, pushed = 0, sent = 0;  // sent: stage phases begun, the end marker's included
  int tile = 0;
  FxTile next{0, 0, 0, 0};
  if (lane == 0) {
    tile = dyn ? atomicAdd(prm.sched, 1) : (int)blockIdx.x;
    if (tile < ntiles) next = prm.dtiles[tile];
  }
  tile = __shfl_sync(0xffffffffu, tile, 0);
  bool ok = true;
  for (;; k++) {
    const int b = k % NST;
    if (k >= NST) {
      if (!mbar_wait_bounded(&empty[b], ((k / NST) - 1) & 1, prm.wait_ns)) {
        if (lane == 0) atomicOr(prm.err, ERR_TMA_TIMEOUT);
        ok = false;
        break;
      }
      if constexpr (EXCH) {  // the tile this stage held is done: to the exchange warp
        if (!xq.push(pushed, tinfo + kFxTileInfoBytes * b, lane, prm)) {
          ok = false;
          break;
        }
        pushed++;
      }
    }
    if (tile >= ntiles) {
      if (lane == 0) {
        tslot[b] = -1;
        mbar_arrive(&full[b]);
      }
      sent = k + 1;
      break;
    }
    if (lane == 0) {
      tslot[b] = tile;
      const int cur = tile;
      const FxTile t = next;
      tile = dyn ? atomicAdd(prm.sched, 1) : tile + (int)gridDim.x;
      if (tile < ntiles) next = prm.dtiles[tile];  // in flight while this tile's loads are issued
      const CUtensorMap* in = prm.dmaps_in + 3 * t.sub;
      const CUtensorMap* na = prm.dmaps_na + 2 * t.sub;
      unsigned char* st = smem + b * Tile::STAGE_BYTES;
      // array coordinates: the interior starts at column HX, row HY
      const int x = t.i0, y = t.j0;
      mbar_arrive_expect_tx(&full[b], Tile::TX_BYTES + kFxTileInfoBytes);
      bulk_copy_g2s(smem + Tile::OFF_TINFO + kFxTileInfoBytes * b, prm.dtinfo + (long long)kFxTileInfoBytes * cur,
                    kFxTileInfoBytes, &full[b]);
      tma_load_3d(st, &in[0], x, y, 2, &full[b]);                     // p: origin (HX + i0 - HX, HY + j0 - HY)
      tma_load_3d(st + Tile::OFF_U, &in[1], x, y + HY, 0, &full[b]);  // u: x halo only
      tma_load_3d(st + Tile::OFF_V, &in[2], x + HX, y, 1, &full[b]);  // v: y halo only
      if (Tile::LOAD_UN) tma_load_3d(st + Tile::OFF_N, &na[0], x + HX, y + HY, 0, &full[b]);
      if (Tile::LOAD_ACC) tma_load_3d(st + Tile::OFF_A, &na[1], x + HX, y + HY, 0, &full[b]);
    }
    tile = __shfl_sync(0xffffffffu, tile, 0);
    issued = sent = k + 1;
  }
  if constexpr (EXCH) {
    // the tiles still held: to the exchange warp after their release; then the end marker
    for (int kk = pushed; ok && kk < issued; kk++) {
      if (!mbar_wait_bounded(&empty[kk % NST], (kk / NST) & 1, prm.wait_ns)) {
        if (lane == 0) atomicOr(prm.err, ERR_TMA_TIMEOUT);
        ok = false;
        break;
      }
      ok = xq.push(pushed, tinfo + kFxTileInfoBytes * (kk % NST), lane, prm);
      pushed += ok;
    }
    if (ok) xq.push(pushed, nullptr, lane, prm);  // else the exchange warp's own wait runs out
  }
  if (lane == 0) {
    // the CTA must not exit with copies in flight
    for (int kk = (sent >= NST ? sent - NST : 0); kk < sent; kk++)
      if (!mbar_wait_bounded(&full[kk % NST], (kk / NST) & 1, prm.wait_ns)) atomicOr(prm.err, ERR_TMA_TIMEOUT);
    if (dyn) {
      __threadfence();
      if (atomicAdd(prm.sched + 1, 1) == (int)gridDim.x - 1) {
        atomicExch(prm.sched, 0);
        atomicExch(prm.sched + 1, 0);
      }
    }
  }
}

// One tile of a fixed-point FP64 stage for the compute warps: tile origin (i0, j0)
// in the arrays' interior indices. The stage's p, u, v boxes hold int64
// (converted by the converter warps); u^n, acc are FP64 point boxes. Closure rows
// and SAT faces follow the global indices I = xoff + i, J = yoff + j (prm.nx,
// prm.ny: the global grid); interior stencils read across subdomain edges from
// the ghost lines the boxes include. `in`, `wout` and the stage's RK4 coefficients
// (c_acc, c_w in true units, fx_ca / fx_cw scaled per component) come from the
// caller: the single grid passes prm's, a batch its instance's for the stage.
// KIND: WK_HOM (rho = K = 1) or WK_CONST (rho = 1, constant K, folded into fx_sigp
// and the p coefficients; the SAT takes K).
template <int ORD, int STAGE, typename Tile, int KIND = WK_HOM>
__device__ __forceinline__ void wave_tile_fixed(const WaveParams<double>& prm, const FxGeom& g, const double* in0,
                                                double* wout, const double c_acc, const double c_w,
                                                const double* fx_ca, const double* fx_cw, const unsigned char* st,
                                                const int i0, const int j0, const int warp, const int lane,
                                                const int ep, const int euv, const bool bad, uint64_t* dbar,
                                                uint32_t* dphase, const int b, const int k) {
  static_assert(KIND == WK_HOM || KIND == WK_CONST, "fixed-point stencils: constant coefficients");
  constexpr int TY = Tile::TY, CS = OpShape<ORD>::CS;
  constexpr int HX = Tile::HX, HY = Tile::HY, PW = Tile::PW;
  constexpr int ROWS = TY / Tile::WARPS;
  constexpr int TPT = TY * kWaveTX;
  const int NX = prm.nx, NY = prm.ny;
  const long long pitch = g.pitch, plane = g.plane;
  const double* in = in0 + g.base;
  const long long* iP = reinterpret_cast<const long long*>(st);
  const long long* iU = reinterpret_cast<const long long*>(st + Tile::OFF_U);
  const long long* iV = reinterpret_cast<const long long*>(st + Tile::OFF_V);
  const double* sN = reinterpret_cast<const double*>(st + Tile::OFF_N);
  const double* sA = reinterpret_cast<const double*>(st + Tile::OFF_A);
  double* sD = reinterpret_cast<double*>(const_cast<unsigned char*>(st) + Tile::OFF_DEF);
  // x faces of the global grid inside this tile (their SAT goes to the deferred pass)
  const int iw = -g.xoff, ie = NX - 1 - g.xoff;  // local indices of global columns 0 and NX - 1
  const bool xfaces = dbar != nullptr && prm.bc != BC_NONE &&
                      ((iw >= i0 && iw < i0 + kWaveTX) || (ie >= i0 && ie < i0 + kWaveTX && ie < g.nx));
  const double sg[3] = {prm.fx_sig[0], prm.fx_sig[1], prm.fx_sigp};
  const int ebp = ep + 11, ebuv = euv + 11;  // fx_to's exponent bases
  (void)sN;
  (void)sA;
#pragma unroll
  for (int rr = 0; rr < ROWS; rr++) {
    const int y = warp * ROWS + rr;
    const int j = j0 + y;
    if (j >= g.ny) continue;
    const int J = g.yoff + j;
    const bool yint = (J >= CS) && (J < NY - CS);
    const long long rowq = (long long)(j + g.row0) * pitch;
#pragma unroll
    for (int cc = 0; cc < kWaveTX / 32; cc++) {
      const int x = lane + 32 * cc;
      const int i = i0 + x;
      if (i >= g.nx) continue;
      const int I = g.xoff + i;
      const bool xint = (I >= CS) && (I < NX - CS);
      const long long* cP = iP + (y + HY) * PW + (x + HX);
      const long long* cU = iU + y * PW + (x + HX);
      const long long* cV = iV + (y + HY) * kWaveTX + x;
      // closure lines start at the global first point of the line (inside the arrays
      // for a subdomain at the physical boundary, which holds a whole closure block)
      const double* xline = in + rowq + g.col0 - g.xoff;
      const double* yline = in + (long long)(g.row0 - g.yoff) * pitch + (i + g.col0);
      // RHS in units of sigma per component: F_u = sx ku, F_v = sy kv, F_p = sx kp
      double ku, kv, kp;
      if (xint) {
        ku = fx_to(fx_stencil<ORD>(cP, 1), ebp);
      } else {
        ku = closure_line<double, ORD>(xline + 2 * plane, 1, NX, I, prm.dx.cls) * prm.fx_isig[0];
      }
      if (yint) {
        kv = fx_to(fx_stencil<ORD>(cP, PW), ebp);
      } else {
        kv = closure_line<double, ORD>(yline + 2 * plane, pitch, NY, J, prm.dy.cls) * prm.fx_isig[1];
      }
      if (xint && yint && prm.fx_square) {
        kp = fx_to(fx_stencil<ORD>(cU, 1) + fx_stencil<ORD>(cV, kWaveTX), ebuv);
      } else {
        const double ax = xint ? fx_to(fx_stencil<ORD>(cU, 1), ebuv)
                               : closure_line<double, ORD>(xline, 1, NX, I, prm.dx.cls) * prm.fx_isig[0];
        const double ay = yint ? fx_to(fx_stencil<ORD>(cV, kWaveTX), ebuv)
                               : closure_line<double, ORD>(yline + plane, pitch, NY, J, prm.dy.cls) * prm.fx_isig[1];
        kp = fma(prm.fx_rho, ay, ax);
      }
      if (bad) ku = kv = kp = __longlong_as_double(0x7FF8000000000000ll);

      const long long q = rowq + i + g.col0;
      const int sp = y * kWaveTX + x;  // point within a 3-component smem box
      const bool edge = (I == 0) || (J == 0) || (I == NX - 1) || (J == NY - 1);
      if (prm.bc != BC_NONE && edge) {
        if (xfaces && J != 0 && J != NY - 1) {
          double* d = sD + ((I == 0 ? 0 : TY) + y) * 3;  // an x-face point only: deferred
          d[0] = ku;
          d[1] = kv;
          d[2] = kp;
          continue;
        }
        // SAT and the stage update in true units
        const double pc = in[2 * plane + q], uc = in[q], vc = in[plane + q];
        const Rhs3<double> r =
            apply_sat<double, KIND>(prm, in, I, J, pc, uc, vc, Rhs3<double>{sg[0] * ku, sg[1] * kv, sg[2] * kp});
        const double kt[3] = {r.u, r.v, r.p};
#pragma unroll
        for (int c = 0; c < 3; c++) {
          const double cen = (STAGE == ST_FIRST) ? sN[c * TPT + sp] : 0.0;
          wave_point_store<double, STAGE, Tile>(prm, wout, c_acc, c_w, sA, sN, nullptr, sp, c,
                                                g.base + c * plane + q, kt[c], cen);
        }
        continue;
      }
      const double kf[3] = {ku, kv, kp};
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const long long o = g.base + c * plane + q;
        if constexpr (STAGE == ST_RHS) {
          prm.kout[o] = sg[c] * kf[c];
        } else {
          const double cen = (STAGE == ST_FIRST) ? sN[c * TPT + sp] : 0.0;
          wave_point_store<double, STAGE, Tile>(prm, wout, fx_ca[c], fx_cw[c], sA, sN, nullptr, sp, c, o,
                                                kf[c], cen);
        }
      }
    }
  }
  if (xfaces) {
    __syncwarp();
    if (lane == 0) mbar_arrive(dbar);  // this warp's deferred entries are in shared memory
    const uint32_t par = (*dphase >> b) & 1u;
    *dphase ^= 1u << b;
    if (warp != k % Tile::WARPS) return;
    if (!mbar_wait_bounded(dbar, par, prm.wait_ns)) {
      if (lane == 0) atomicOr(prm.err, ERR_TMA_TIMEOUT);
      return;
    }
    for (int e = lane; e < 2 * TY; e += 32) {
      const int side = e / TY, y = e - side * TY, j = j0 + y;
      const int I = side == 0 ? 0 : NX - 1, i = I - g.xoff, J = g.yoff + j;
      if (i < i0 || i >= i0 + kWaveTX || i >= g.nx || j >= g.ny || J == 0 || J == NY - 1) continue;
      const int x = i - i0;
      const long long q = (long long)(j + g.row0) * pitch + i + g.col0;
      const double pc = in[2 * plane + q], uc = in[q], vc = in[plane + q];
      const double* d = sD + (side * TY + y) * 3;
      const Rhs3<double> r =
          apply_sat<double, KIND>(prm, in, I, J, pc, uc, vc, Rhs3<double>{sg[0] * d[0], sg[1] * d[1], sg[2] * d[2]});
      const double kt[3] = {r.u, r.v, r.p};
      const int sp = y * kWaveTX + x;
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const double cen = (STAGE == ST_FIRST) ? sN[c * TPT + sp] : 0.0;
        wave_point_store<double, STAGE, Tile>(prm, wout, c_acc, c_w, sA, sN, nullptr, sp, c,
                                              g.base + c * plane + q, kt[c], cen);
      }
    }
  }
}

// Converter warps: the p, u and v boxes of one ring stage to int64 in place.
// t is the thread's index among the converter threads. The exponent maxima go
// through one barrier among the converters (fxa, bounded wait): each converter
// warp writes its own p and u/v maxima to wmax[warp][0..1], every converter then
// takes the maximum over them, and so does every compute warp later (fx_tile_emax),
// so nothing has to be reset between tiles. Returns false if the wait ran out.
template <typename Tile>
__device__ __forceinline__ bool fx_convert_stage(unsigned char* st, uint64_t* fxa, int* wmax, uint32_t parity,
                                                 unsigned long long wait_ns, int t);

// The p and u/v exponent maxima of a converted stage from its converter warps'
// pairs, with the tile guard applied: a box whose maximum is below 64 (values
// under 2^-959) converts to zeros, and one at 2031 or more (values from 2^1008,
// Inf, NaN) marks the tile bad.
template <int CONV>
__device__ __forceinline__ void fx_tile_emax(const int* wmax, int& ep, int& euv, bool& bad) {
  ep = 0;
  euv = 0;
#pragma unroll
  for (int c = 0; c < CONV; c++) {
    ep = max(ep, wmax[2 * c]);
    euv = max(euv, wmax[2 * c + 1]);
  }
  bad = ep >= 2031 || euv >= 2031;
  if (ep < 64) ep = 2111;  // every value converts to 0
  if (euv < 64) euv = 2111;
}

template <typename Tile>
__device__ __forceinline__ bool fx_convert_stage(unsigned char* st, uint64_t* fxa, int* wmax, uint32_t parity,
                                                 unsigned long long wait_ns, int t) {
  constexpr int NT = 32 * Tile::CONV;
  constexpr int NP = Tile::PH * Tile::PW, NU = Tile::TY * Tile::PW, NV = Tile::PH * kWaveTX;
  uint2* wP = reinterpret_cast<uint2*>(st);
  uint2* wU = reinterpret_cast<uint2*>(st + Tile::OFF_U);
  uint2* wV = reinterpret_cast<uint2*>(st + Tile::OFF_V);
  const int lane = t & 31, cw = t >> 5;
  unsigned mp = 0, muv = 0;
  for (int e = t; e < NP; e += NT) mp = max(mp, wP[e].y & 0x7FF00000u);
  for (int e = t; e < NU; e += NT) muv = max(muv, wU[e].y & 0x7FF00000u);
  for (int e = t; e < NV; e += NT) muv = max(muv, wV[e].y & 0x7FF00000u);
  mp = __reduce_max_sync(0xffffffffu, mp);
  muv = __reduce_max_sync(0xffffffffu, muv);
  if (lane == 0) {
    wmax[2 * cw] = (int)(mp >> 20);
    wmax[2 * cw + 1] = (int)(muv >> 20);
  }
  __syncwarp();
  if (lane == 0) mbar_arrive(fxa);
  if (!mbar_wait_bounded(fxa, parity, wait_ns)) return false;
  int ep, euv;
  bool bad;
  fx_tile_emax<Tile::CONV>(wmax, ep, euv, bad);
  (void)bad;
  long long* iP = reinterpret_cast<long long*>(wP);
  long long* iU = reinterpret_cast<long long*>(wU);
  long long* iV = reinterpret_cast<long long*>(wV);
#pragma unroll 4
  for (int e = t; e < NP; e += NT) {
    const uint2 w = wP[e];
    iP[e] = fx_from(w.x, w.y, ep);
  }
#pragma unroll 4
  for (int e = t; e < NU; e += NT) {
    const uint2 w = wU[e];
    iU[e] = fx_from(w.x, w.y, euv);
  }
#pragma unroll 4
  for (int e = t; e < NV; e += NT) {
    const uint2 w = wV[e];
    iV[e] = fx_from(w.x, w.y, euv);
  }
  // the converted boxes were written through the generic proxy; order those writes
  // before the TMA (async proxy) refills the stage
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  return true;
}

// A fixed-point FP64 stage with warp roles: WARPS compute warps, CONV converter
// warps and one producer warp. Per ring stage: the producer's TMA loads complete
// `full` (1 arrival + bytes), the converters convert the stage's boxes and arrive on
// `conv` (CONV arrivals), the compute warps evaluate the tile and arrive on
// `empty` (WARPS arrivals), which lets the producer refill the stage. Conversion
// of the next tile thus overlaps the computation of the current one, and the
// compute warps meet no barrier but the deferred x-face pass. Every wait is
// bounded (prm.wait_ns); a wait that runs out sets the error word and the warp
// stops, so the others' waits run out in turn.
template <int ORD, int STAGE, bool DEC = false>
__global__ void __launch_bounds__(fx_kernel_threads<WaveStageTile<double, ORD, WK_HOM, STAGE>, DEC>(), 1)
    wave_fixed_kernel(const __grid_constant__ CUtensorMap mapP, const __grid_constant__ CUtensorMap mapU,
                      const __grid_constant__ CUtensorMap mapV, const __grid_constant__ CUtensorMap mapN,
                      const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapC,
                      const __grid_constant__ CUtensorMap mapK, const __grid_constant__ WaveParams<double> prm) {
  using Tile = WaveStageTile<double, ORD, WK_HOM, STAGE>;
  constexpr int TY = Tile::TY, NST = Tile::NST, WARPS = Tile::WARPS, CONV = Tile::CONV;
  static_assert(CONV >= 1, "the converter-warp kernel needs converter warps");
  extern __shared__ __align__(128) unsigned char smem[];
  if (prm.fx_sig[0] == 0.0 || prm.fx_sig[1] == 0.0) {  // the host did not set the fixed-point scales
    if (threadIdx.x == 0) atomicOr(prm.err, ERR_BAD_LAUNCH);
    return;
  }
  if (prm.skip && *prm.skip) return;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + Tile::OFF_BAR);
  uint64_t* empty = full + NST;
  uint64_t* dbar = reinterpret_cast<uint64_t*>(smem + Tile::OFF_DBAR);
  int* tslot = reinterpret_cast<int*>(smem + Tile::OFF_BAR + 192);
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
    if constexpr (DEC) {
      const FxExchangeQueue<Tile> xq(smem);
      for (int s = 0; s < FxExchangeQueue<Tile>::SLOTS; s++) {
        mbar_init(&xq.full[s], 1);
        mbar_init(&xq.empty[s], 1);
      }
    }
    fence_barrier_init();
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntx = (prm.nx + kWaveTX - 1) / kWaveTX;

  if (warp == WARPS + CONV) {
    if constexpr (DEC)
      decomp_produce<Tile, STAGE>(prm, smem, full, empty, tslot, FxExchangeQueue<Tile>(smem), lane);
    else if (lane == 0)
      wave_produce<Tile>(mapP, mapU, mapV, mapN, mapA, mapC, mapK, prm, smem, full, empty, tslot,
                         prm.sched != nullptr);
    return;
  }
  if constexpr (DEC) {
    if (warp == WARPS + CONV + 1) {  // the exchange warp
      if constexpr (STAGE == ST_FIRST || STAGE == ST_MID || STAGE == ST_LAST)
        decomp_exchange<Tile, STAGE>(prm, FxExchangeQueue<Tile>(smem), lane);
      return;
    }
  }
  if (warp >= WARPS) {
    // ---------------- converters
    const int t = threadIdx.x - 32 * WARPS;
    for (int k = 0;; k++) {
      const int b = k % NST;
      if (!mbar_wait_bounded(&full[b], (k / NST) & 1, prm.wait_ns)) {
        if (lane == 0) atomicOr(prm.err, ERR_TMA_TIMEOUT);
        break;
      }
      const int tile = tslot[b];
      if (tile >= 0 && !fx_convert_stage<Tile>(smem + b * Tile::STAGE_BYTES, &fxa[b], wmax + 16 * b, (k / NST) & 1,
                                                prm.wait_ns, t)) {
        if (lane == 0) atomicOr(prm.err, ERR_TMA_TIMEOUT);
        break;
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&conv[b]);  // converted, or the end marker passed on
      if (tile < 0) break;
    }
    return;
  }
  // ---------------- compute warps
  uint32_t dphase = 0;  // parity of each stage's next deferred-pass barrier phase
  for (int k = 0;; k++) {
    const int b = k % NST;
    if (!mbar_wait_bounded(&conv[b], (k / NST) & 1, prm.wait_ns)) {
      if (lane == 0) atomicOr(prm.err, ERR_TMA_TIMEOUT);
      break;
    }
    const int tile = tslot[b];
    if (tile < 0) break;
    int i0, j0;
    FxGeom g;
    if constexpr (DEC) {
      const FxTileInfo* info = reinterpret_cast<const FxTileInfo*>(smem + Tile::OFF_TINFO + kFxTileInfoBytes * b);
      g = info->g;
      i0 = info->i0;
      j0 = info->j0;
    } else {
      i0 = (tile % ntx) * kWaveTX;
      j0 = (tile / ntx) * TY;
      g = FxGeom{prm.nx, prm.ny, 0, 0, 0, 0, prm.pitch, prm.plane, 0};
    }
    int ep, euv;
    bool bad;
    fx_tile_emax<CONV>(wmax + 16 * b, ep, euv, bad);
    wave_tile_fixed<ORD, STAGE, Tile>(prm, g, prm.in, prm.wout, prm.c_acc, prm.c_w, prm.fx_ca, prm.fx_cw,
                                      smem + b * Tile::STAGE_BYTES, i0, j0, warp, lane, ep, euv, bad, &dbar[b], &dphase,
                                      b, k);
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[b]);
  }
}

}  // namespace sbp
