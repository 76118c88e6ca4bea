// wave2d.cuh -- fused RHS + SAT + RK4-stage kernel for the 2D first-order
// acoustic wave system (u, v, p):
//   F_u = -(1/rho) D1x p,  F_v = -(1/rho) D1y p,  F_p = -K (D1x u + D1y v)
// with the reference's operators (code/include/sbpops/D1_central.h) and its
// region split (code/include/partitioned_rhs/rhs.h:373-398): closure rows for
// the first/last cls_sz lines of each direction, the central stencil between.
//
// Persistent, warp-specialised pipeline. One CTA per SM walks the tiles of
// the grid (TX x TY points each) in a fixed stride. The last warp is the
// producer: its lane 0 issues the TMA loads of tile k+1 into a ring of
// shared-memory stages while the consumer warps (8 to 16 per kind and
// precision) compute tile k from another:
//   * the stage input with halos: p with an x and y halo, u with an x halo,
//     v with a y halo (the star stencil needs no corners of u, v);
//   * the per-point RK4 operands the stage needs, each as one 3-component
//     box: u^n and acc for stages 2-3, acc for stage 4, plus u^n and the
//     Kahan term for the FP32 stage 4.
//   * variable coefficients: [1/rho | K] as one 2-component box.
// Consumers touch global memory only for their outputs (coalesced streaming
// stores), for closure-row taps (boundary strips) and for the FP64 copies of
// the coefficients at boundary points. The SAT of x-face points runs in a
// separate pass per tile (see wave_tile_compute).
// Every mbarrier wait is bounded by %globaltimer; a timeout sets an error bit
// that the host reads and the CTA stops after letting its copies land.
//
// State layout in HBM: structure of arrays, component planes [u | v | p],
// each ny rows of `pitch` elements (pitch a multiple of 64).
#pragma once

#include "rkf_tableau.cuh"
#include "sbp_device.cuh"

namespace sbp {

enum WaveKind : int { WK_HOM = 0, WK_VAR = 1, WK_MMS = 2, WK_CONST = 3 };  // WK_CONST: rho = 1, K = kconst
enum BcKind : int { BC_NONE = 0, BC_FREE_SURFACE = 1, BC_CHARACTERISTIC = 2 };
enum Stage : int { ST_RHS = 0, ST_FIRST = 1, ST_MID = 2, ST_LAST = 4, ST_RKF1 = 11, ST_RKF6 = 16 };
// ST_RKF1 + s - 1 (s = 1..6): stage s of the Runge-Kutta-Fehlberg 4(5) attempt (FP64):
// k_s, then the input of stage s+1 (s < 6) or the candidate solution and the
// error partial sum (s = 6).
constexpr bool is_rkf_stage(int stage) { return stage >= ST_RKF1 && stage <= ST_RKF6; }

// The constant-coefficient FP64 stages (RHS and RK4; rho = K = 1) evaluate their
// interior stencils in exact integer arithmetic (wave2d_fixed.cuh) instead of
// FP64 FMAs, which GB300 issues at about 1/64 of its FP32 rate. The build may set
// SBP_FP64_FIXED=0 to compare with the FP64 tap chains.
#ifndef SBP_FP64_FIXED
#define SBP_FP64_FIXED 1
#endif
template <typename T, int KIND, int STAGE> constexpr bool wave_fixed() {
  return SBP_FP64_FIXED != 0 && sizeof(T) == 8 && KIND == WK_HOM && !is_rkf_stage(STAGE);
}

struct FxSub;   // a subdomain of a decomposed grid (wave2d_fixed.cuh)
struct FxTile;  // a tile of a decomposed grid (wave2d_fixed.cuh)

template <typename T> struct WaveParams {
  int nx, ny;
  long long pitch;    // elements per row
  long long plane;    // elements per component plane (ny * pitch)
  const T* in;        // stage input state (3 planes); closure taps are read here
  T* un;              // u^n (3 planes); written in place by ST_LAST
  T* acc;             // RK4 accumulator (3 planes)
  T* wout;            // next stage input (3 planes)
  T* kout;            // ST_RHS output (3 planes)
  T* comp;            // FP32: compensation term of the summed update (3 planes)
  const T* rinv;      // WK_VAR: 1/rho (1 plane)
  const T* kmod;      // WK_VAR: K (1 plane)
  const double* rho64;  // WK_VAR: rho in FP64, read at boundary points
  const double* k64;    // WK_VAR: K in FP64, read at boundary points
  DirTaps<T> dx, dy;  // -hix * stencils, -hiy * stencils
  double bwx, bwy;    // hix * HI[0], hiy * HI[0]: SAT weights (FP64)
  T c_acc, c_w;       // acc (+)= c_acc * k ; w = u^n + c_w * k
  T kconst;           // WK_CONST: bulk modulus K (rho = 1)
  double kz, kc;      // WK_CONST: sqrt(K) in FP64, the impedance and speed of the characteristic SAT
  double dt;          // batched: the instance's time step
  int bc;             // BcKind
  int ysplit;         // 0: one block; else rows [0,ysplit) and [ysplit,ny) are two blocks
                      // sharing an interface line (WK_VAR only)
  double t, xl0, xl1, hix, hiy;  // WK_MMS: stage time and grid geometry
  const double* tctl;  // the adaptive integrator's (t, h); WK_MMS stage time tctl[0] + tc * tctl[1]
  double tc;
  const int* skip;     // non-null and set: the kernel returns at entry
  T* rkk[6];           // ST_RKF*: stage derivatives k_1..k_6 (3 planes each)
  const T* rku;        // ST_RKF*: the attempt's starting state u
  T* rkunew;           // ST_RKF6: candidate solution u5
  double* rkpart;      // ST_RKF6: one error partial sum per CTA
  double rkatol, rkrtol;
  int* err;
  // Bounded waits: limit of every mbarrier wait in ns (0: kWaitLimitNs). Test
  // aid for that path: test_drop_tile = k + 1 makes the producer issue no load
  // for tile k, so the consumers' wait for it runs out (0: none).
  unsigned long long wait_ns;
  int test_drop_tile;
  // Fixed-point FP64 stages (wave_fixed): the RHS is formed in units of
  // sigma = -hi/den per direction (den: the interior stencil's common denominator),
  // fx_isig = 1/sigma, fx_rho = sigma_y/sigma_x, fx_square = (sigma_x == sigma_y),
  // fx_sigp = the p equation's scale (sigma_x, times K for a constant K != 1),
  // and fx_ca/fx_cw are c_acc/c_w times the scale of each component (u: sigma_x,
  // v: sigma_y, p: fx_sigp).
  double fx_sig[2], fx_isig[2], fx_rho, fx_sigp;
  double fx_ca[3], fx_cw[3];
  int fx_square;
  // Dynamic tile queue: sched[0] hands out tile indices, sched[1] counts the CTAs
  // done; the last CTA resets both to zero for the next launch. Null: each CTA
  // walks the tiles with a fixed stride (the Fehlberg stages always do, so their
  // per-CTA error partials keep a fixed summation order).
  int* sched;
  // Decomposed grid (wave_fixed_kernel<.., true>): the tile list, the subdomains,
  // and per subdomain the TMA maps of the stage input's p, u, v boxes ([sub][3])
  // and the point maps of u^n and acc ([sub][2]), all in device memory.
  const FxTile* dtiles;
  const FxSub* dsubs;
  const unsigned char* dtinfo;  // per tile its FxTileInfo block (kFxTileInfoBytes each)
  const CUtensorMap* dmaps_in;
  const CUtensorMap* dmaps_na;
  int dntiles;
};

constexpr int kWaveTX = 64;            // tile width (x, contiguous)
constexpr int kWaveConsumerWarps = 8;  // compute warps where no kind- or form-specific count is set
constexpr int kWaveThreads = 32 * (kWaveConsumerWarps + 1);

// FP32 keeps the state with a Kahan-compensated final update.
template <typename T> struct IsCompensated { static constexpr bool value = false; };
template <> struct IsCompensated<float> { static constexpr bool value = true; };

// Tile geometry and shared-memory plan for (T, order, stage). The x halo is
// rounded up so that (tile origin - halo) * sizeof(T) is a multiple of 16
// bytes (TMA rule for the innermost coordinate); tile origins are multiples of 64.
template <typename T> constexpr int default_wave_ty() { return sizeof(T) == 8 ? 16 : 32; }

// Pipeline shape of the single-instance kernel for FP32 (tile rows, ring depth);
// the build may override them to compare shapes.
#ifndef SBP_FP32_TILE_ROWS
#define SBP_FP32_TILE_ROWS 32
#endif
#ifndef SBP_FP32_RING
#define SBP_FP32_RING 2
#endif

// Pipeline shape of the constant-coefficient FP64 kernel (tile rows, consumer
// warps); the build may override them to compare shapes. Measured with the
// fixed-point stencils at 4096^2, order 4 (point-stage updates/s), with the dynamic
// tile queue: compute warps converting their own tiles (12, 12) 3.76e10, (16, 16)
// 4.20e10, (20, 20) 4.43e10, (22, 22) 4.56e10; a third ring stage (12, 12) 3.74e10;
// with converter warps (SBP_FP64_CONV) overlapping the conversion of the next tile:
// (22, 22) 5.11e10 (4 converters) / 5.18e10 (6), and, with the shared memory of a
// third ring stage, (12, 12) 5.39e10 (4), (14, 14) 5.63e10 (4) / 5.67e10 (6).
#ifndef SBP_FP64_TILE_ROWS
#define SBP_FP64_TILE_ROWS 14
#endif
#ifndef SBP_FP64_WARPS
#define SBP_FP64_WARPS 14
#endif

// Tile height of the single-instance kernel: the variable-coefficient FP32
// kind also stages 1/rho and K, so it uses 24 rows to keep two stages in 227 KB.
template <typename T, int KIND> constexpr int wave_ty() {
  return sizeof(T) == 8 ? (KIND == WK_HOM ? SBP_FP64_TILE_ROWS : 16) : (KIND == WK_VAR ? 24 : SBP_FP32_TILE_ROWS);
}
// Shared-memory ring depth (tiles in flight + the one being computed).
#ifndef SBP_FP64_RING
#define SBP_FP64_RING 3
#endif
// Converter warps of the fixed-point FP64 stages: they convert tile k+1 to int64
// while the compute warps work on tile k (0: the compute warps convert each tile
// themselves, between two barriers).
#ifndef SBP_FP64_CONV
#define SBP_FP64_CONV 6
#endif
// The first and last stages of the constant-coefficient FP64 kernel load one point box
// less than the middle stages, which leaves room for a fourth ring stage (4096^2, order 4:
// 5.73e10 against 5.64e10 point-stage updates/s with three; 8 converter warps instead of
// 6 measured slower with either depth, 1024^2 unchanged).
#ifndef SBP_FP64_RING_FL
#define SBP_FP64_RING_FL 4
#endif
template <typename T, int KIND, int STAGE = ST_MID> constexpr int wave_ring() {
  return (sizeof(T) == 4 && KIND != WK_VAR)
             ? SBP_FP32_RING
             : (sizeof(T) == 8 && KIND == WK_HOM ? ((STAGE == ST_FIRST || STAGE == ST_LAST) ? SBP_FP64_RING_FL
                                                                                            : SBP_FP64_RING)
                                                 : 2);
}
// Consumer warps of the single-instance kernel. The variable-coefficient and
// manufactured-solution FP64 kernels need up to 166 registers a thread, which
// leaves room for 8 warps; the constant-coefficient FP64 kernels (at most 128)
// run 12 with one tile row each, the constant-coefficient FP32 kernels 16 with
// two rows each (more warps hide more load latency).
#ifndef SBP_FP32_WARPS
#define SBP_FP32_WARPS 16
#endif
// The variable-coefficient FP32 kernel (up to 124 registers) runs 12 warps on its
// 24-row tiles: 2.20 s against 2.54 s with 8 for 1748 steps at 4096^2.
#ifndef SBP_FP32_VAR_WARPS
#define SBP_FP32_VAR_WARPS 12
#endif
// Where the variable-coefficient kernels read 1/rho and K: 1 from the tile's
// TMA box in shared memory, 0 with read-only global loads (no box), 2 both
// (the box loaded but unused; kept to measure what the box costs).
#ifndef SBP_VAR_COEF
#define SBP_VAR_COEF 1
#endif
template <typename T, int KIND> constexpr int wave_warps() {
  return sizeof(T) == 4 ? (KIND != WK_VAR ? SBP_FP32_WARPS : SBP_FP32_VAR_WARPS)
                        : (KIND == WK_HOM ? SBP_FP64_WARPS : kWaveConsumerWarps);
}

template <typename T, int ORD, int STAGE, int TY_ = default_wave_ty<T>(), int PRM_BYTES = 0, bool COEF = false,
          int NST_ = 2, int WARPS_ = kWaveConsumerWarps, bool FIX_ = false, int CONV_ = 0>
struct WaveTile {
  static constexpr int WARPS = WARPS_;                        // consumer (compute) warps
  static constexpr int CONV = CONV_;                          // fixed-point stages: converter warps
  static constexpr int THREADS = 32 * (WARPS_ + CONV_ + 1);   // + the producer warp
  static constexpr bool COMP = IsCompensated<T>::value;
  static constexpr int TY = TY_;                              // tile height
  static constexpr int R = (OpShape<ORD>::W - 1) / 2;
  static constexpr int HXA = 16 / sizeof(T);
  static constexpr int HX = ((R + HXA - 1) / HXA) * HXA;     // x halo loaded
  static constexpr int HY = R;                                // y halo loaded
  static constexpr int PW = kWaveTX + 2 * HX;                 // p/u tile row length
  static constexpr int PH = TY + 2 * HY;                      // p/v tile rows
  static constexpr bool FIX = FIX_;  // fixed-point FP64 stage: the p/u/v boxes become int64 in place
  // u^n as a point box: the stages that read it, and the fixed-point first stage, whose
  // stencil boxes no longer hold the doubles of u^n once converted
  // (Reading u^n and acc with streaming loads instead of point boxes, to free shared
  // memory for taller tiles, measured slower: 22 rows 4.23e10 against 4.56e10 point-stage
  // updates/s at 4096^2, 31 rows with 31 warps 4.55e10.)
  static constexpr bool LOAD_UN = (STAGE == ST_MID) || (STAGE == ST_LAST && COMP) || (FIX_ && STAGE == ST_FIRST);
  static constexpr bool LOAD_ACC = (STAGE == ST_MID) || (STAGE == ST_LAST);
  static constexpr bool LOAD_COMP = (STAGE == ST_LAST && COMP);
  static constexpr bool LOAD_COEF = COEF;  // 1/rho and K planes as one 2-component point box
  static constexpr int align128(int b) { return (b + 127) / 128 * 128; }
  static constexpr int BYTES_P = PH * PW * (int)sizeof(T);
  static constexpr int BYTES_U = TY * PW * (int)sizeof(T);
  static constexpr int BYTES_V = PH * kWaveTX * (int)sizeof(T);
  static constexpr int BYTES_PT = 3 * TY * kWaveTX * (int)sizeof(T);  // one 3-component point box
  static constexpr int OFF_U = align128(BYTES_P);
  static constexpr int OFF_V = OFF_U + align128(BYTES_U);
  static constexpr int OFF_N = OFF_V + align128(BYTES_V);
  static constexpr int OFF_A = OFF_N + (LOAD_UN ? BYTES_PT : 0);
  static constexpr int OFF_C = OFF_A + (LOAD_ACC ? BYTES_PT : 0);
  static constexpr int BYTES_K = 2 * TY * kWaveTX * (int)sizeof(T);
  static constexpr int OFF_K = align128(OFF_C + (LOAD_COMP ? BYTES_PT : 0));
  static constexpr int OFF_PRM = align128(OFF_K + (LOAD_COEF ? BYTES_K : 0));  // batched: instance parameters
  // the RHS of the tile's x-face points, kept for the deferred SAT pass ([side][row][u, v, p])
  static constexpr int OFF_DEF = OFF_PRM + align128(PRM_BYTES);
  static constexpr int STAGE_BYTES = OFF_DEF + align128(2 * TY * 3 * (int)sizeof(T));
  static constexpr int NST = NST_;                            // ring depth
  static constexpr int OFF_BAR = NST * STAGE_BYTES;           // full[NST], empty[NST]
  static constexpr int OFF_DBAR = OFF_BAR + 128;              // deferred-pass barriers[NST]
  // + 192: the tile index of each stage (int[NST]; -1 marks the end)
  // Fixed-point stages, at OFF_FX: barriers[8] "exponent maxima known" (+0) and
  // "boxes converted" (+64), then per stage the p and u/v exponent maxima: one pair
  // per converter warp (int[8][8][2], +128) when converter warps convert, or one
  // shared pair (int[8][2]) when the compute warps do.
  static constexpr int OFF_FX = OFF_BAR + 256;
  // Decomposed grids: eight 192-byte slots of tile geometry (that of its subdomain's
  // neighbours included): one per ring stage, the rest the exchange queue; then the
  // exchange queue's barriers (full[8] at +0, empty[8] at +64)
  static constexpr int OFF_TINFO = OFF_FX + 640;
  static constexpr int OFF_XBAR = OFF_TINFO + 8 * 192;
  static constexpr int SMEM = OFF_BAR + 256 + (FIX_ ? 640 + 8 * 192 + 128 : 0);
  static constexpr uint32_t TX_BYTES = BYTES_P + BYTES_U + BYTES_V + (LOAD_UN ? BYTES_PT : 0) +
                                       (LOAD_ACC ? BYTES_PT : 0) + (LOAD_COMP ? BYTES_PT : 0) +
                                       (LOAD_COEF ? BYTES_K : 0) + PRM_BYTES;
  static_assert(TY % WARPS == 0, "tile rows must split evenly over the consumer warps");
  static_assert(CONV <= 8, "converter warps");
  static_assert(NST >= 2 && NST <= 8, "ring depth");
  static_assert(SMEM <= 227 * 1024, "wave tile pipeline exceeds shared memory");
};

// Closure row of D1 along one line: left block for i < CS, mirrored negated
// block for i >= n - CS (D1_central.h:57-65, :95-104), scaled taps.
template <typename T, int ORD>
__device__ __forceinline__ T closure_line(const T* __restrict__ line, long long st, int n, int i,
                                          const T (&cls)[6][9]) {
  constexpr int CW = OpShape<ORD>::CW;
  T s;
  if (i < OpShape<ORD>::CS) {
    s = cls[i][0] * __ldg(line);
#pragma unroll
    for (int k = 1; k < CW; k++) s = fma(cls[i][k], __ldg(line + k * st), s);
  } else {
    const int r = n - 1 - i;
    const T* base = line + (long long)(n - CW) * st;
    s = -cls[r][CW - 1] * __ldg(base);
#pragma unroll
    for (int k = 1; k < CW; k++) s = fma(-cls[r][CW - 1 - k], __ldg(base + k * st), s);
  }
  return s;
}

// Closure row of D1 along a line held in shared memory: closure_line's operations
// in its order (the same bits), with plain loads.
template <typename T, int ORD>
__device__ __forceinline__ T closure_line_smem(const T* line, int st, int n, int i, const T (&cls)[6][9]) {
  constexpr int CW = OpShape<ORD>::CW;
  T s;
  if (i < OpShape<ORD>::CS) {
    s = cls[i][0] * line[0];
#pragma unroll
    for (int k = 1; k < CW; k++) s = fma(cls[i][k], line[k * st], s);
  } else {
    const int r = n - 1 - i;
    const T* base = line + (n - CW) * st;
    s = -cls[r][CW - 1] * base[0];
#pragma unroll
    for (int k = 1; k < CW; k++) s = fma(-cls[r][CW - 1 - k], base[k * st], s);
  }
  return s;
}

// A closure row from global memory, for the rare points whose closure stencil leaves
// their tile's boxes; out of line, so its registers stay out of the kernels' main loops.
template <typename T, int ORD>
__device__ __noinline__ T closure_line_global(const T* line, long long st, int n, int i, const T (&cls)[6][9]) {
  return closure_line<T, ORD>(line, st, n, i, cls);
}

__device__ __forceinline__ double mms_x(double xl, int i, double hi) { return xl + (double)i / hi; }

template <typename T> struct Rhs3 { T u, v, p; };

// SAT boundary terms at a boundary point, FP64 weights, in the reference's
// order west, south, east, north. Kept out of line so interior points branch
// around it instead of issuing its FP64 instructions under a predicate.
template <typename T, int KIND>
__device__ __noinline__ Rhs3<T> apply_sat(const WaveParams<T>& prm, const T* in, int i, int j, T pc, T uc, T vc,
                                          Rhs3<T> k) {
  const int nx = prm.nx, ny = prm.ny;
  double rho = 1.0, kk = 1.0;
  if constexpr (KIND == WK_VAR) {
    rho = prm.rho64[(long long)j * nx + i];
    kk = prm.k64[(long long)j * nx + i];
  } else if constexpr (KIND == WK_CONST) {
    kk = (double)prm.kconst;
  }
  const double p64 = (double)pc;
  double ku64 = (double)k.u, kv64 = (double)k.v, kp64 = (double)k.p;
  if (prm.bc == BC_NONE) {
    // matrix-free apply only
  } else if (prm.bc == BC_FREE_SURFACE) {
    // free_surface_bc_* (code/demo/wave_hom/wave_eq_hom_rhs.h:389-441); rho^-1 for WK_VAR
    const double ri = (KIND == WK_VAR) ? 1.0 / rho : 1.0;
    if (i == 0) ku64 = (KIND == WK_VAR) ? ku64 - ri * (prm.bwx * p64) : ku64 - prm.bwx * p64;
    if (j == 0) kv64 = (KIND == WK_VAR) ? kv64 - ri * (prm.bwy * p64) : kv64 - prm.bwy * p64;
    if (i == nx - 1) ku64 = (KIND == WK_VAR) ? ku64 + ri * (prm.bwx * p64) : ku64 + prm.bwx * p64;
    if (j == ny - 1) kv64 = (KIND == WK_VAR) ? kv64 + ri * (prm.bwy * p64) : kv64 + prm.bwy * p64;
  } else {
    // characteristic SAT on the incoming characteristic p + Z u_n; WK_CONST reads
    // Z = c = sqrt(K) from the parameters (computed once on the host: an FP64
    // square root per boundary point is long on the FP64 pipe)
    const double z = KIND == WK_CONST ? prm.kz : sqrt(rho * kk);
    const double c = KIND == WK_CONST ? prm.kc : sqrt(kk / rho);
    const double hr = 0.5 / rho, hc = 0.5 * c;
    const double u64 = (double)uc, v64 = (double)vc;
    if (i == 0) { const double g = prm.bwx * (p64 + z * u64); ku64 -= hr * g; kp64 -= hc * g; }
    if (j == 0) { const double g = prm.bwy * (p64 + z * v64); kv64 -= hr * g; kp64 -= hc * g; }
    if (i == nx - 1) { const double g = prm.bwx * (p64 - z * u64); ku64 += hr * g; kp64 -= hc * g; }
    if (j == ny - 1) { const double g = prm.bwy * (p64 - z * v64); kv64 += hr * g; kp64 -= hc * g; }
  }
  if constexpr (KIND == WK_VAR) {
    // Interface line between the two blocks: energy-conserving SAT on the jumps
    // of p and v (Carpenter, Nordstrom & Gottlieb 1999): lower block
    // F_v += w/(2 rho) [p], F_p += w K/2 [v]; upper block with the opposite sign.
    const int ys = prm.ysplit;
    if (ys > 0 && prm.bc != BC_NONE && (j == ys - 1 || j == ys)) {
      const int jo = (j == ys - 1) ? ys : ys - 1;  // the other block's copy of the line
      const long long qo = (long long)jo * prm.pitch + i;
      const double po = (double)in[2 * prm.plane + qo], vo = (double)in[prm.plane + qo];
      const double s = (j == ys - 1) ? 1.0 : -1.0;
      kv64 += s * (0.5 / rho) * (prm.bwy * (p64 - po));
      kp64 += s * (0.5 * kk) * (prm.bwy * ((double)vc - vo));
    }
  }
  return Rhs3<T>{(T)ku64, (T)kv64, (T)kp64};
}

// RK4 stage update of component c of one point (o: its offset in the state,
// sp: its place in a tile's 3-component point boxes).
template <typename T, int STAGE, typename Tile>
__device__ __forceinline__ void wave_point_store(const WaveParams<T>& prm, T* wout, const T c_acc, const T c_w,
                                                 const T* sA, const T* sN, const T* sC, int sp, int c, long long o,
                                                 T kc, T cen) {
  constexpr int TPT = Tile::TY * kWaveTX;
  if constexpr (STAGE == ST_RHS) {
    prm.kout[o] = kc;
  } else if constexpr (STAGE == ST_FIRST) {
    // acc = u + dt/6 k1 (FP32 compensated: acc = dt/6 k1), w = u + dt/2 k1
    st_stream(prm.acc + o, Tile::COMP ? c_acc * kc : fma(c_acc, kc, cen));
    st_stream(wout + o, fma(c_w, kc, cen));
  } else if constexpr (STAGE == ST_MID) {
    st_stream(prm.acc + o, fma(c_acc, kc, sA[c * TPT + sp]));
    st_stream(wout + o, fma(c_w, kc, sN[c * TPT + sp]));
  } else if constexpr (STAGE == ST_LAST) {
    const T d = fma(c_acc, kc, sA[c * TPT + sp]);
    if constexpr (Tile::COMP) {
      // Kahan summation of the step increment into the FP32 state
      const T u0 = sN[c * TPT + sp], e = sC[c * TPT + sp];
      const T yv = d - e;
      const T tv = u0 + yv;
      st_stream(prm.comp + o, (tv - u0) - yv);
      st_stream(prm.un + o, tv);
    } else {
      st_stream(prm.un + o, d);
    }
  }
}

// Fehlberg stage S = STAGE - ST_RKF1 + 1 of component c of one point: the same
// sums, in the same order, as the unfused combination kernels (rk45.cu). kS is
// this stage's derivative, pre[0..S-2] = k_1..k_{S-1} and pre[S-1] = u (S > 1).
template <typename T, int STAGE, int NPRE>
__device__ __forceinline__ void wave_point_rkf(const WaveParams<T>& prm, T* wout, long long o, double kS, double cen,
                                               const double (&pre)[NPRE], double* errsq) {
  constexpr int S = STAGE - ST_RKF1 + 1;
  const double h = prm.tctl[1];
  if constexpr (S < 6) {
    prm.rkk[S - 1][o] = kS;
    double s = kRkfA[S][0] * (S == 1 ? kS : pre[0]);
#pragma unroll
    for (int jj = 1; jj < S; jj++) s = fma(kRkfA[S][jj], jj == S - 1 ? kS : pre[jj], s);
    const double u0 = S == 1 ? cen : pre[S - 1];
    st_stream(wout + o, fma(h, s, u0));
  } else {
    double u5, u4;
    rkf_candidate(pre[5], h, pre[0], pre[2], pre[3], pre[4], kS, u5, u4);
    st_stream(prm.rkunew + o, u5);
    *errsq += rkf_err_term(u5, u4, prm.rkatol, prm.rkrtol);
  }
}

// k_1..k_{S-1} and u of one component of one point for Fehlberg stage S (stage 6
// does not need k2: its weights are zero).
template <typename T, int RKS>
__device__ __forceinline__ void wave_rkf_preload(const WaveParams<T>& prm, long long o, double (&pre)[RKS]) {
  if constexpr (RKS > 1) {
#pragma unroll
    for (int jj = 0; jj < RKS - 1; jj++)
      if (RKS < 6 || jj != 1) pre[jj] = __ldg(prm.rkk[jj] + o);
    pre[RKS - 1] = __ldg(prm.rku + o);
  }
}

// One tile of the stage for the consumer warps: everything the tile needs is
// in the shared-memory stage `st` (laid out as Tile), except closure-row taps
// and coefficient fields. `in` is the stage input, `wout` the next stage input.
template <typename T, int ORD, int KIND, int STAGE, typename Tile>
__device__ __forceinline__ void wave_tile_compute(const WaveParams<T>& prm, const T* __restrict__ in, T* wout,
                                                  const T c_acc, const T c_w, const unsigned char* st, const int i0,
                                                  const int j0, const int warp, const int lane,
                                                  double* errsq = nullptr, uint64_t* dbar = nullptr,
                                                  uint32_t* dphase = nullptr, const int b = 0, const int k = 0) {
  constexpr bool COMP = Tile::COMP;
  constexpr int TY = Tile::TY, W = OpShape<ORD>::W, CS = OpShape<ORD>::CS, R = Tile::R;
  constexpr int HX = Tile::HX, HY = Tile::HY, PW = Tile::PW;
  constexpr int ROWS = TY / Tile::WARPS;
  // FP64 is bound by the FP64 pipe: unrolling the warp's rows gives more
  // independent FMA chains. FP32 is bound by HBM and runs faster rolled.
  constexpr int ROW_UNROLL = sizeof(T) == 8 ? ROWS : 1;
  constexpr int TPT = TY * kWaveTX;  // points per tile (one component)
  const int nx = prm.nx, ny = prm.ny;
  const long long pitch = prm.pitch, plane = prm.plane;
  const T* sP = reinterpret_cast<const T*>(st);
  const T* sU = reinterpret_cast<const T*>(st + Tile::OFF_U);
  const T* sV = reinterpret_cast<const T*>(st + Tile::OFF_V);
  const T* sN = reinterpret_cast<const T*>(st + Tile::OFF_N);
  const T* sA = reinterpret_cast<const T*>(st + Tile::OFF_A);
  const T* sC = reinterpret_cast<const T*>(st + Tile::OFF_C);
  const T* sK = reinterpret_cast<const T*>(st + Tile::OFF_K);  // [1/rho | K] when Tile::LOAD_COEF
  // Deferred SAT: a point on an x face only (not on a y face or the interface
  // lines) leaves its RHS in the stage's deferred box and skips SAT and update;
  // after every consumer warp has passed the tile's rows, one warp applies the
  // SAT and the update to all of them, one point per lane. In a row warp a single
  // x-face lane would hold the FP64 pipe for the whole SAT sequence.
  constexpr bool DEFER_OK = true;  // every stage kind, Fehlberg stages included
  const bool xfaces = DEFER_OK && dbar != nullptr && prm.bc != BC_NONE &&
                      (i0 == 0 || (nx - 1 >= i0 && nx - 1 < i0 + kWaveTX));
  T* sD = reinterpret_cast<T*>(const_cast<unsigned char*>(st) + Tile::OFF_DEF);
  (void)sD;
  (void)sN;
  (void)sA;
  (void)sC;
  (void)sK;
  // Closure lines come from the boxes where their stencil lies inside them (box columns
  // i0 - HX .. i0 + 63 + HX, rows j0 - HY .. j0 + TY - 1 + HY), else from global memory:
  // the first CW points of a line when the tile starts it, the last CW when they start no
  // earlier and end no later than the box. The same values either way.
  constexpr int CW = OpShape<ORD>::CW;
  const bool xl_in = i0 == 0, xr_in = nx - CW >= i0 - HX && nx <= i0 + kWaveTX + HX;
#pragma unroll ROW_UNROLL
  for (int rr = 0; rr < ROWS; rr++) {
    const int y = warp * ROWS + rr;
    const int j = j0 + y;
    if (j >= ny) continue;
    // block-local row (two-block problems: the interface rows close each block)
    const int jb0 = (prm.ysplit > 0 && j >= prm.ysplit) ? prm.ysplit : 0;
    const int nyb = (prm.ysplit > 0) ? (j >= prm.ysplit ? ny - prm.ysplit : prm.ysplit) : ny;
    const int jl = j - jb0;
    const bool yint = (jl >= CS) && (jl < nyb - CS);
    const int yb = jl < CS ? jb0 : jb0 + nyb - CW;  // the first row of this point's y closure stencil
    const bool y_in = yb >= j0 - HY && yb + CW <= j0 + TY + HY;
#pragma unroll
    for (int cc = 0; cc < kWaveTX / 32; cc++) {
      const int x = lane + 32 * cc;
      const int i = i0 + x;
      if (i >= nx) continue;
      const bool xint = (i >= CS) && (i < nx - CS);
      const T* rowP = sP + (y + HY) * PW + (x + HX - R);
      const T* rowU = sU + y * PW + (x + HX - R);
      const T* colP = sP + y * PW + (x + HX);   // row y+HY-R
      const T* colV = sV + y * kWaveTX + x;     // row y+HY-R
      const T pc = rowP[R], uc = rowU[R], vc = colV[R * kWaveTX];
      // Fehlberg stages: the point's u and k_1..k_{S-1} are loaded here, ahead of
      // the stencil arithmetic, so that their latency overlaps it (stage 6 does
      // not need k2: its weights are zero).
      constexpr int RKS = is_rkf_stage(STAGE) ? STAGE - ST_RKF1 + 1 : 1;
      double rkpre[3][RKS];  // [c][0..RKS-2] = k_1..k_{RKS-1}, [c][RKS-1] = u (RKS > 1)
      if constexpr (RKS > 1) {
        const long long q0 = (long long)j * pitch + i;
#pragma unroll
        for (int c = 0; c < 3; c++) wave_rkf_preload<T, RKS>(prm, c * plane + q0, rkpre[c]);
      }
      (void)rkpre;

      T dxp, dyp, kp;
      if (xint) {
        dxp = prm.dx.taps[0] * rowP[0];
#pragma unroll
        for (int s = 1; s < W; s++)
          if (s != R) dxp = fma(prm.dx.taps[s], rowP[s], dxp);
      } else if (i < CS ? xl_in : xr_in) {
        dxp = closure_line_smem<T, ORD>(sP + (y + HY) * PW + (HX - i0), 1, nx, i, prm.dx.cls);
      } else {
        dxp = closure_line_global<T, ORD>(in + 2 * plane + (long long)j * pitch, 1, nx, i, prm.dx.cls);
      }
      if (yint) {
        dyp = prm.dy.taps[0] * colP[0];
#pragma unroll
        for (int s = 1; s < W; s++)
          if (s != R) dyp = fma(prm.dy.taps[s], colP[s * PW], dyp);
      } else if (y_in) {
        dyp = closure_line_smem<T, ORD>(sP + (jb0 - j0 + HY) * PW + (x + HX), PW, nyb, jl, prm.dy.cls);
      } else {
        dyp = closure_line_global<T, ORD>(in + 2 * plane + (long long)jb0 * pitch + i, pitch, nyb, jl, prm.dy.cls);
      }
      if (xint) {
        kp = prm.dx.taps[0] * rowU[0];
#pragma unroll
        for (int s = 1; s < W; s++)
          if (s != R) kp = fma(prm.dx.taps[s], rowU[s], kp);
      } else if (i < CS ? xl_in : xr_in) {
        kp = closure_line_smem<T, ORD>(sU + y * PW + (HX - i0), 1, nx, i, prm.dx.cls);
      } else {
        kp = closure_line_global<T, ORD>(in + (long long)j * pitch, 1, nx, i, prm.dx.cls);
      }
      if (yint) {
#pragma unroll
        for (int s = 0; s < W; s++)
          if (s != R) kp = fma(prm.dy.taps[s], colV[s * kWaveTX], kp);
      } else if (y_in) {
        kp += closure_line_smem<T, ORD>(sV + (jb0 - j0 + HY) * kWaveTX + x, kWaveTX, nyb, jl, prm.dy.cls);
      } else {
        kp += closure_line_global<T, ORD>(in + plane + (long long)jb0 * pitch + i, pitch, nyb, jl, prm.dy.cls);
      }

      const long long q = (long long)j * pitch + i;
      T ku, kv;
      if constexpr (KIND == WK_HOM) {
        ku = dxp;
        kv = dyp;
      } else if constexpr (KIND == WK_CONST) {
        ku = dxp;
        kv = dyp;
        kp = prm.kconst * kp;
      } else if constexpr (KIND == WK_VAR) {
        T ri, km;
        if constexpr (SBP_VAR_COEF == 1) {  // the tile's [1/rho | K] box
          ri = sK[y * kWaveTX + x];
          km = sK[TPT + y * kWaveTX + x];
        } else {
          ri = __ldg(prm.rinv + q);
          km = __ldg(prm.kmod + q);
        }
        ku = ri * dxp;
        kv = ri * dyp;
        kp = km * kp;
      } else {  // WK_MMS (FP64): code/demo/wave/wave_eq_rhs.h:42-64
        const double PI = 3.14159265358979323846264;
        const double xx = mms_x(prm.xl0, i, prm.hix), yy = mms_x(prm.xl1, j, prm.hiy);
        const double ri = 1. / (2 + xx * yy);
        const double ts = prm.tctl ? __dadd_rn(prm.tctl[0], __dmul_rn(prm.tc, prm.tctl[1])) : prm.t;
        const double ct = cos(5 * PI * ts);
        const double fu = -(3 * PI * ct * cos(3 * PI * xx) * sin(4 * PI * yy) * (xx * yy + 1)) / (xx * yy + 2);
        const double fv = -(4 * PI * ct * cos(4 * PI * yy) * sin(3 * PI * xx) * (xx * yy + 1)) / (xx * yy + 2);
        ku = (T)(ri * (double)dxp + fu);
        kv = (T)(ri * (double)dyp + fv);
      }

      // SAT boundary terms (boundary points only)
      const bool edge = (i == 0) || (j == 0) || (i == nx - 1) || (j == ny - 1) ||
                        (prm.ysplit > 0 && (j == prm.ysplit - 1 || j == prm.ysplit));
      if (prm.bc != BC_NONE && edge) {
        if (xfaces && j != 0 && j != ny - 1 && !(prm.ysplit > 0 && (j == prm.ysplit - 1 || j == prm.ysplit))) {
          T* d = sD + ((i == 0 ? 0 : TY) + y) * 3;  // an x-face point only: deferred
          d[0] = ku;
          d[1] = kv;
          d[2] = kp;
          continue;
        }
        const Rhs3<T> r = apply_sat<T, KIND>(prm, in, i, j, pc, uc, vc, Rhs3<T>{ku, kv, kp});
        ku = r.u;
        kv = r.v;
        kp = r.p;
      }

      // RK4 stage update (classical RK4, code/include/time_stepping/time_stepping.h:127-142)
      const T kc[3] = {ku, kv, kp};
      const T cen[3] = {uc, vc, pc};
      const int sp = y * kWaveTX + x;  // point within a 3-component smem box
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const long long o = c * plane + q;
        if constexpr (STAGE == ST_RHS) {
          prm.kout[o] = kc[c];
        } else if constexpr (is_rkf_stage(STAGE)) {
          wave_point_rkf<T, STAGE, RKS>(prm, wout, o, (double)kc[c], (double)cen[c], rkpre[c], errsq);
        } else {
          wave_point_store<T, STAGE, Tile>(prm, wout, c_acc, c_w, sA, sN, sC, sp, c, o, kc[c], cen[c]);
        }
      }
    }
  }
  if constexpr (DEFER_OK) {
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
        const int i = side == 0 ? 0 : nx - 1;
        if (i < i0 || i >= i0 + kWaveTX || j >= ny || j == 0 || j == ny - 1 ||
            (prm.ysplit > 0 && (j == prm.ysplit - 1 || j == prm.ysplit)))
          continue;
        const int x = i - i0;
        const T pc = sP[(y + HY) * PW + x + HX], uc = sU[y * PW + x + HX], vc = sV[(y + HY) * kWaveTX + x];
        const T* d = sD + (side * TY + y) * 3;
        const Rhs3<T> r = apply_sat<T, KIND>(prm, in, i, j, pc, uc, vc, Rhs3<T>{d[0], d[1], d[2]});
        const T kc[3] = {r.u, r.v, r.p};
        const T cen[3] = {uc, vc, pc};
        const long long q = (long long)j * pitch + i;
        const int sp = y * kWaveTX + x;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          if constexpr (is_rkf_stage(STAGE)) {
            constexpr int RKS = STAGE - ST_RKF1 + 1;
            double pre[RKS];
            wave_rkf_preload<T, RKS>(prm, c * plane + q, pre);
            wave_point_rkf<T, STAGE, RKS>(prm, wout, c * plane + q, (double)kc[c], (double)cen[c], pre, errsq);
          } else {
            wave_point_store<T, STAGE, Tile>(prm, wout, c_acc, c_w, sA, sN, sC, sp, c, c * plane + q, kc[c], cen[c]);
          }
        }
      }
    }
  }
}

// The Tile type of the single-instance kernel for (T, order, kind, stage).
template <typename T, int ORD, int KIND, int STAGE>
using WaveStageTile = WaveTile<T, ORD, STAGE, wave_ty<T, KIND>(), 0, KIND == WK_VAR && SBP_VAR_COEF != 0,
                               wave_ring<T, KIND, STAGE>(), wave_warps<T, KIND>(), wave_fixed<T, KIND, STAGE>(),
                               wave_fixed<T, KIND, STAGE>() ? SBP_FP64_CONV : 0>;

// The producer (one lane): takes the CTA's tiles, from the dynamic queue or with a
// fixed stride, writes each tile's index into its ring stage and issues the stage's
// TMA loads; a stage holding -1, completed without bytes, marks the end. Waits for
// every copy it issued before it returns, then counts the CTA done in the queue.
template <typename Tile, typename T>
__device__ __forceinline__ void wave_produce(const CUtensorMap& mapP, const CUtensorMap& mapU, const CUtensorMap& mapV,
                                             const CUtensorMap& mapN, const CUtensorMap& mapA, const CUtensorMap& mapC,
                                             const CUtensorMap& mapK, const WaveParams<T>& prm, unsigned char* smem,
                                             uint64_t* full, uint64_t* empty, int* tslot, bool dyn) {
  constexpr int TY = Tile::TY, HX = Tile::HX, HY = Tile::HY, NST = Tile::NST;
  const int ntx = (prm.nx + kWaveTX - 1) / kWaveTX;
  const int ntiles = ntx * ((prm.ny + TY - 1) / TY);
  prefetch_tensormap(&mapP);
  int k = 0;
  int tile = dyn ? atomicAdd(prm.sched, 1) : (int)blockIdx.x;
  for (;; k++) {
    const int b = k % NST;
    if (k >= NST && !mbar_wait_bounded(&empty[b], ((k / NST) - 1) & 1, prm.wait_ns)) {
      atomicOr(prm.err, ERR_TMA_TIMEOUT);
      break;
    }
    if (tile >= ntiles) {  // the end marker: a phase completed without bytes
      tslot[b] = -1;
      mbar_arrive(&full[b]);
      k++;
      break;
    }
    tslot[b] = tile;
    const int cur = tile;
    // the next index is fetched now: the atomic's latency overlaps this tile's loads
    tile = dyn ? atomicAdd(prm.sched, 1) : tile + (int)gridDim.x;
    if (cur + 1 == prm.test_drop_tile) continue;  // no load: the consumers' wait runs out
    unsigned char* st = smem + b * Tile::STAGE_BYTES;
    const int i0 = (cur % ntx) * kWaveTX, j0 = (cur / ntx) * TY;
    mbar_arrive_expect_tx(&full[b], Tile::TX_BYTES);
    tma_load_3d(st, &mapP, i0 - HX, j0 - HY, 2, &full[b]);
    tma_load_3d(st + Tile::OFF_U, &mapU, i0 - HX, j0, 0, &full[b]);
    tma_load_3d(st + Tile::OFF_V, &mapV, i0, j0 - HY, 1, &full[b]);
    if (Tile::LOAD_UN) tma_load_3d(st + Tile::OFF_N, &mapN, i0, j0, 0, &full[b]);
    if (Tile::LOAD_ACC) tma_load_3d(st + Tile::OFF_A, &mapA, i0, j0, 0, &full[b]);
    if (Tile::LOAD_COMP) tma_load_3d(st + Tile::OFF_C, &mapC, i0, j0, 0, &full[b]);
    if (Tile::LOAD_COEF) tma_load_3d(st + Tile::OFF_K, &mapK, i0, j0, 0, &full[b]);
  }
  // the CTA must not exit with copies in flight: wait for the last NST stages
  for (int kk = (k >= NST ? k - NST : 0); kk < k; kk++)
    if (!mbar_wait_bounded(&full[kk % NST], (kk / NST) & 1, prm.wait_ns)) atomicOr(prm.err, ERR_TMA_TIMEOUT);
  if (dyn) {  // every CTA has stopped taking tiles when the last one gets here
    __threadfence();
    if (atomicAdd(prm.sched + 1, 1) == (int)gridDim.x - 1) {
      atomicExch(prm.sched, 0);
      atomicExch(prm.sched + 1, 0);
    }
  }
}

}  // namespace sbp

#include "wave2d_fixed.cuh"

namespace sbp {

template <typename T, int ORD, int KIND, int STAGE>
__global__ void __launch_bounds__(32 * (wave_warps<T, KIND>() + 1), 1)
    wave_stage_kernel(const __grid_constant__ CUtensorMap mapP, const __grid_constant__ CUtensorMap mapU,
                      const __grid_constant__ CUtensorMap mapV, const __grid_constant__ CUtensorMap mapN,
                      const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapC,
                      const __grid_constant__ CUtensorMap mapK, const __grid_constant__ WaveParams<T> prm) {
  using Tile = WaveStageTile<T, ORD, KIND, STAGE>;
  constexpr int TY = Tile::TY, HX = Tile::HX, HY = Tile::HY, NST = Tile::NST, WARPS = Tile::WARPS;
  extern __shared__ __align__(128) unsigned char smem[];
  if (prm.skip && *prm.skip) return;  // uniform over the grid: set before this launch
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + Tile::OFF_BAR);
  uint64_t* empty = full + NST;

  const int nx = prm.nx, ny = prm.ny;
  const int ntx = (nx + kWaveTX - 1) / kWaveTX;
  const int ntiles = ntx * ((ny + TY - 1) / TY);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  uint64_t* dbar = reinterpret_cast<uint64_t*>(smem + Tile::OFF_DBAR);
  uint64_t* fxa = reinterpret_cast<uint64_t*>(smem + Tile::OFF_FX);       // fixed: exponent maxima known
  uint64_t* fxb = fxa + 8;                                                 // fixed: boxes converted
  int* fxmax = reinterpret_cast<int*>(smem + Tile::OFF_FX + 128);          // fixed: [NST][2] maxima
  if constexpr (Tile::FIX) {
    if (prm.fx_sig[0] == 0.0 || prm.fx_sig[1] == 0.0) {  // the host did not set the fixed-point scales
      if (threadIdx.x == 0) atomicOr(prm.err, ERR_BAD_LAUNCH);
      return;
    }
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], WARPS);
      mbar_init(&dbar[s], WARPS);
      if constexpr (Tile::FIX) {
        mbar_init(&fxa[s], WARPS);
        mbar_init(&fxb[s], WARPS);
        fxmax[2 * s] = fxmax[2 * s + 1] = 0;
      }
    }
    fence_barrier_init();
  }
  __syncthreads();

  int* tslot = reinterpret_cast<int*>(smem + Tile::OFF_BAR + 192);
  const bool dyn = prm.sched != nullptr && !is_rkf_stage(STAGE);

  if (warp == WARPS) {
    if (lane == 0) wave_produce<Tile>(mapP, mapU, mapV, mapN, mapA, mapC, mapK, prm, smem, full, empty, tslot, dyn);
    return;
  }

  // ---------------- consumers: warps 0 .. WARPS-1
  double errsq = 0.0;  // ST_RKF6: this thread's share of the weighted error sum
  uint32_t dphase = 0;  // parity of each stage's next deferred-pass barrier phase
  for (int k = 0;; k++) {
    const int b = k % NST;
    if (!mbar_wait_bounded(&full[b], (k / NST) & 1, prm.wait_ns)) {
      if (lane == 0) atomicOr(prm.err, ERR_TMA_TIMEOUT);
      break;
    }
    const int tile = tslot[b];
    if (tile < 0) break;
    const int i0 = (tile % ntx) * kWaveTX, j0 = (tile / ntx) * TY;
    if constexpr (Tile::FIX) {
      int emax[2];
      bool bad;
      if (!fx_convert_tile<Tile>(smem + b * Tile::STAGE_BYTES, &fxa[b], &fxb[b], fxmax + 2 * b, (k / NST) & 1,
                                 prm.wait_ns, threadIdx.x, emax, bad)) {
        if (lane == 0) atomicOr(prm.err, ERR_TMA_TIMEOUT);
        break;
      }
      const FxGeom g{prm.nx, prm.ny, 0, 0, 0, 0, prm.pitch, prm.plane, 0};
      wave_tile_fixed<ORD, STAGE, Tile>(prm, g, prm.in, prm.wout, prm.c_acc, prm.c_w, prm.fx_ca, prm.fx_cw,
                                        smem + b * Tile::STAGE_BYTES, i0, j0, warp, lane, emax[0], emax[1], bad,
                                        &dbar[b], &dphase, b, k);
      // the converted boxes were written through the generic proxy; order those writes
      // before the TMA (async proxy) refills the stage
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    } else {
      wave_tile_compute<T, ORD, KIND, STAGE, Tile>(prm, prm.in, prm.wout, prm.c_acc, prm.c_w,
                                                   smem + b * Tile::STAGE_BYTES, i0, j0, warp, lane, &errsq, &dbar[b],
                                                   &dphase, b, k);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[b]);
  }
  if constexpr (STAGE == ST_RKF6) {
    // fixed-order sum over the consumer threads -> one partial per CTA
    __shared__ double warp_sum[WARPS];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) errsq += __shfl_down_sync(0xffffffffu, errsq, off);
    if (lane == 0) warp_sum[warp] = errsq;
    asm volatile("bar.sync 1, %0;" ::"n"(32 * WARPS) : "memory");  // consumer warps only
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int q = 0; q < WARPS; q++) s += warp_sum[q];
      prm.rkpart[blockIdx.x] = s;
    }
  }
}

}  // namespace sbp
