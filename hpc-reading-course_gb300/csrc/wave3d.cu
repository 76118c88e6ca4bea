// wave3d.cu -- fused RHS + SAT + RK4-stage kernels of the 3D acoustic wave
// system (wave3d.cuh), orders 2, 4 and 6, FP64 or compensated FP32.
//
// Two forms. The plane-ring kernel (the default for both precisions) stages each z
// plane of the block's column tile in shared memory with 16-byte cp.async copies
// running ahead of the plane it computes, so its loads are in flight while it
// computes; measured at 256^3, order 4: FP32 6.35e10 point-stage updates/s (0.67
// of the measured HBM copy bandwidth) against 3.48e10 for the column kernel, FP64
// 1.32e10 against 1.22e10 (FP64-pipe bound). The column kernel (one thread per
// (i, j) column marching 16 planes, every tap a read-only global load) runs where
// the ring kernel's 32-bit offsets or 16-byte alignment do not hold.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>

#include "launch.h"

namespace sbp {

constexpr int kW3X = 64, kW3Y = 4, kW3Z = 16;

// Boundary terms on the faces the point lies on (FP64 arithmetic, as the 2D kernels):
// free surface (wave_eq_hom_rhs.h:389-441 per face): lower face F_ud -= bw_d p, upper F_ud += bw_d p;
// characteristic (Z = c = 1): lower face g = bw_d (p + u_d): F_ud -= g/2, F_p -= g/2;
// upper face g = bw_d (p - u_d): F_ud += g/2, F_p -= g/2.
template <typename T> struct Rhs4 { T u, v, w, p; };

template <typename T>
__device__ __noinline__ Rhs4<T> wave3d_sat(const Wave3Params<T>& prm, int i, int j, int k, T uc, T vc, T wc, T pc,
                                           Rhs4<T> kc) {
  // values and results by value: a noinline function taking arrays by reference
  // would keep the caller's arrays in local memory on every point. Only the
  // components a face changes go through FP64 (the others would round-trip
  // exactly), in the order of the faces, so that a point on one face costs about
  // ten FP64-pipe instructions.
  const T cen[3] = {uc, vc, wc};
  T f[3] = {kc.u, kc.v, kc.w};
  const int idx[3] = {i, j, k};
  const int n[3] = {prm.nx, prm.ny, prm.nz};
  const double p = (double)pc;
  double fp = (double)kc.p;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const bool lo = idx[d] == 0, hi = idx[d] == n[d] - 1;
    if (!lo && !hi) continue;
    const double ud = (double)cen[d];
    double fd = (double)f[d];
    if (prm.bc == BC_CHARACTERISTIC) {
      if (lo) {
        const double g = prm.bw[d] * (p + ud);
        fd -= 0.5 * g;
        fp -= 0.5 * g;
      }
      if (hi) {
        const double g = prm.bw[d] * (p - ud);
        fd += 0.5 * g;
        fp -= 0.5 * g;
      }
    } else {
      if (lo) fd -= prm.bw[d] * p;
      if (hi) fd += prm.bw[d] * p;
    }
    f[d] = (T)fd;
  }
  return Rhs4<T>{f[0], f[1], f[2], (T)fp};
}

// FP64: the z neighbours of p and w come from a per-thread register window (one new
// value of each per plane instead of the five taps); measured at 256^3, order 4:
// 1.209e10 against 1.170e10 point-stages/s. FP32 runs faster without it (3.48e10
// against 3.25e10: at its 40-register budget the window spills).
template <typename T> constexpr bool w3_zwin() { return sizeof(T) == 8; }

// Interior D1 over W values of a register window, in d1_line's order.
template <typename T, int ORD>
__device__ __forceinline__ T taps_window(const DirTaps<T>& d, const T (&c)[OpShape<ORD>::W]) {
  constexpr int W = OpShape<ORD>::W, R = (W - 1) / 2;
  T s = d.taps[0] * c[0];
#pragma unroll
  for (int q = 1; q < W; q++)
    if (q != R) s = fma(d.taps[q], c[q], s);
  return s;
}

// Where the stage update reads acc, u^n and the Kahan term: global memory (column
// kernel) or the shared-memory copies of the ring kernel.
template <typename T> struct GlobalExtras {
  const Wave3Params<T>& prm;
  long long q;
  __device__ __forceinline__ T acc(int c) const { return prm.acc[c * prm.plane + q]; }
  __device__ __forceinline__ T un(int c) const { return prm.un[c * prm.plane + q]; }
  __device__ __forceinline__ T comp(int c) const { return prm.comp[c * prm.plane + q]; }
};

// SAT terms on the faces the point lies on, then the RK stage update of the four
// components at offset q (the same for both kernels).
template <typename T, int STAGE, typename I, typename Ex>
__device__ __forceinline__ void wave3d_finish(const Wave3Params<T>& prm, int i, int j, int k, I q, T (&kc)[4],
                                              const T (&cen)[4], const Ex& ex) {
  const I plane = (I)prm.plane;
  if (prm.bc != BC_NONE &&
      (i == 0 || j == 0 || k == 0 || i == prm.nx - 1 || j == prm.ny - 1 || k == prm.nz - 1)) {
    const Rhs4<T> r = wave3d_sat<T>(prm, i, j, k, cen[0], cen[1], cen[2], cen[3], Rhs4<T>{kc[0], kc[1], kc[2], kc[3]});
    kc[0] = r.u;
    kc[1] = r.v;
    kc[2] = r.w;
    kc[3] = r.p;
  }
  // RK4 stage update (classical RK4, code/include/time_stepping/time_stepping.h:127-142)
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const I o = c * plane + q;
    if constexpr (STAGE == ST_RHS) {
      prm.kout[o] = kc[c];
    } else if constexpr (STAGE == ST_FIRST) {
      st_stream(prm.acc + o, prm.compensated ? prm.c_acc * kc[c] : fma(prm.c_acc, kc[c], cen[c]));
      st_stream(prm.wout + o, fma(prm.c_w, kc[c], cen[c]));
    } else if constexpr (STAGE == ST_MID) {
      st_stream(prm.acc + o, fma(prm.c_acc, kc[c], ex.acc(c)));
      st_stream(prm.wout + o, fma(prm.c_w, kc[c], ex.un(c)));
    } else {  // ST_LAST
      const T d = fma(prm.c_acc, kc[c], ex.acc(c));
      if (prm.compensated) {
        const T u0 = ex.un(c), e = ex.comp(c);
        const T yv = d - e;
        const T tv = u0 + yv;
        prm.comp[o] = (tv - u0) - yv;
        prm.un[o] = tv;
      } else {
        prm.un[o] = d;
      }
    }
  }
}

template <typename T, int ORD, int STAGE>
__device__ __forceinline__ void wave3d_point(const Wave3Params<T>& prm, int i, int j, int k,
                                             const T (&pw)[OpShape<ORD>::W], const T (&ww)[OpShape<ORD>::W]) {
  const int nx = prm.nx, ny = prm.ny, nz = prm.nz;
  const long long pitch = prm.pitch, slab = prm.slab, plane = prm.plane;
  const T* __restrict__ U = prm.in;
  const T* __restrict__ V = U + plane;
  const T* __restrict__ W = V + plane;
  const T* __restrict__ P = W + plane;
  const long long xo = (long long)k * slab + (long long)j * pitch;  // start of the x line
  const long long yo = (long long)k * slab + i;                     // start of the y line (stride pitch)
  const long long zo = (long long)j * pitch + i;                    // start of the z line (stride slab)
  const long long q = xo + i;
  T kc[4];
  kc[0] = d1_line<T, ORD>(P + xo, 1, nx, i, prm.dx);
  kc[1] = d1_line<T, ORD>(P + yo, pitch, ny, j, prm.dy);
  constexpr int CS = OpShape<ORD>::CS;
  const bool zwin = w3_zwin<T>() && k >= CS && k < nz - CS;
  kc[2] = zwin ? taps_window<T, ORD>(prm.dz, pw) : d1_line<T, ORD>(P + zo, slab, nz, k, prm.dz);
  kc[3] = d1_line<T, ORD>(U + xo, 1, nx, i, prm.dx) + d1_line<T, ORD>(V + yo, pitch, ny, j, prm.dy) +
          (zwin ? taps_window<T, ORD>(prm.dz, ww) : d1_line<T, ORD>(W + zo, slab, nz, k, prm.dz));
  const T cen[4] = {__ldg(U + q), __ldg(V + q), __ldg(W + q), __ldg(P + q)};
  wave3d_finish<T, STAGE>(prm, i, j, k, q, kc, cen, GlobalExtras<T>{prm, q});
}

// Blocks per SM the register budget is sized for: the kernel is latency-bound, so
// occupancy pays (measured at 256^3, order 4: FP64 1.02e10 / 1.14e10 / 1.17e10
// point-stages/s at 2 / 3 / 4 blocks, flat beyond; FP32 1.48e10 / 2.10e10 /
// 2.67e10 / 3.07e10 / 3.48e10 at 2 .. 6).
#ifndef SBP_W3_BLOCKS_F64
#define SBP_W3_BLOCKS_F64 4
#endif
#ifndef SBP_W3_BLOCKS_F32
#define SBP_W3_BLOCKS_F32 6
#endif
template <typename T, int ORD, int STAGE>
__global__ void __launch_bounds__(kW3X * kW3Y, sizeof(T) == 8 ? SBP_W3_BLOCKS_F64 : SBP_W3_BLOCKS_F32)
    wave3d_stage_kernel(const __grid_constant__ Wave3Params<T> prm) {
  if (prm.skip && *prm.skip) return;
  const int i = blockIdx.x * kW3X + threadIdx.x;
  const int j = blockIdx.y * kW3Y + threadIdx.y;
  if (i >= prm.nx || j >= prm.ny) return;
  const int k0 = blockIdx.z * kW3Z;
  const int k1 = k0 + kW3Z < prm.nz ? k0 + kW3Z : prm.nz;
  constexpr int W = OpShape<ORD>::W, R = (W - 1) / 2;
  T pw[W], ww[W];  // p and w at planes k - R .. k + R of this column (zero outside the grid)
  const long long zo = (long long)j * prm.pitch + i;
  const T* Pz = prm.in + 3 * prm.plane + zo;
  const T* Wz = prm.in + 2 * prm.plane + zo;
  if constexpr (w3_zwin<T>()) {
#pragma unroll
    for (int s = 0; s < W; s++) {
      const int kk = k0 - R + s;
      const bool in = kk >= 0 && kk < prm.nz;
      pw[s] = in ? __ldg(Pz + kk * prm.slab) : T(0);
      ww[s] = in ? __ldg(Wz + kk * prm.slab) : T(0);
    }
  }
#pragma unroll 1
  for (int k = k0; k < k1; k++) {
    T pn = T(0), wn = T(0);
    const int kn = k + 1 + R;
    if (w3_zwin<T>() && kn < prm.nz && k + 1 < k1) {  // the window's next plane, loaded ahead
      pn = __ldg(Pz + kn * prm.slab);
      wn = __ldg(Wz + kn * prm.slab);
    }
    wave3d_point<T, ORD, STAGE>(prm, i, j, k, pw, ww);
    if constexpr (w3_zwin<T>()) {
#pragma unroll
      for (int s = 0; s + 1 < W; s++) {
        pw[s] = pw[s + 1];
        ww[s] = ww[s + 1];
      }
      pw[W - 1] = pn;
      ww[W - 1] = wn;
    }
  }
}

// Plane-ring form: a block of kR3X x kR3Y threads owns a column tile and marches
// kR3Z planes. The block copies plane m into shared memory with 16-byte cp.async
// chunks (L2 only): p with x and y halos and w into ring A, u with an x halo, v
// with a y halo and the arrays the stage update reads (acc, u^n, the Kahan term)
// into ring B; the x halo is one 16-byte chunk per side. The
// copies run kR3D planes ahead of the plane being computed, so a block keeps
// kR3D planes of loads in flight without holding them in registers (the column
// kernel's bound is the bytes a thread can keep in flight). The z taps of p and w
// read ring A's planes k - R .. k + R. One barrier per plane: ring A has 2R + D + 2
// slots and ring B D + 2, so a copy never lands in a slot that a thread one plane
// behind may still read. Points within CS of a face (closure rows) read their
// lines from global memory as the column kernel does; the interior sums its taps
// in d1_line's order, so both forms give the same values.
#ifndef SBP_R3_X
#define SBP_R3_X 32
#endif
#ifndef SBP_R3_Y
#define SBP_R3_Y 4
#endif
#ifndef SBP_R3_Z
#define SBP_R3_Z 12
#endif
#ifndef SBP_R3_D
#define SBP_R3_D 1
#endif

// Blocks per SM the registers are sized for. Measured at 256^3, order 4, FP32
// (point-stage updates/s): 32 x 8 threads, 3 blocks 5.35e10; 32 x 4, 6 blocks
// 6.22e10, 8 blocks 6.35e10; 64 x 4, 4 blocks 5.68e10; 32 x 2, 12 blocks 6.06e10;
// planes per block 8 / 12 / 16 at 32 x 4: 6.22e10 / 6.22e10 / 5.99e10.
#ifndef SBP_R3_BLOCKS
#define SBP_R3_BLOCKS 8
#endif
#ifndef SBP_R3_BLOCKS_F64
#define SBP_R3_BLOCKS_F64 3
#endif
constexpr int kR3X = SBP_R3_X, kR3Y = SBP_R3_Y, kR3Z = SBP_R3_Z, kR3D = SBP_R3_D;
constexpr int kR3Threads = kR3X * kR3Y;

template <typename T, int ORD, int STAGE> struct Ring3 {
  static constexpr int R = (OpShape<ORD>::W - 1) / 2;
  static constexpr int TX = kR3X, TY = kR3Y, D = kR3D;
  static constexpr int V = 16 / (int)sizeof(T);           // elements per 16-byte copy
  static constexpr int HX = (R + V - 1) / V * V;          // x halo: whole 16-byte chunks
  static constexpr int PX = TX + 2 * HX, PY = TY + 2 * R;  // p and u tiles: PX columns
  // arrays the stage update reads: acc and u^n (ST_MID), plus the Kahan term (ST_LAST)
  static constexpr int NEX = STAGE == ST_MID ? 8 : (STAGE == ST_LAST ? 12 : 0);
  static constexpr int SA = 2 * R + D + 2, SB = D + 2;
  static constexpr int A_W = PY * PX, A_SZ = A_W + TY * TX;  // ring A slot: p tile, then w
  static constexpr int B_V = TY * PX, B_X = B_V + PY * TX;   // ring B slot: u tile, v tile, extras
  static constexpr int B_SZ = B_X + NEX * TY * TX;
  static constexpr size_t SMEM = (size_t)(SA * A_SZ + SB * B_SZ) * sizeof(T);
  static_assert(TX % V == 0 && A_W % V == 0 && A_SZ % V == 0 && B_V % V == 0 && B_X % V == 0 && B_SZ % V == 0,
                "16-byte copies need 16-byte aligned tile rows");
};

// One 16-byte global -> shared copy, not cached in L1.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

// Copies an NR x NC-chunk box of one plane (rows gj0.., columns gi0.. in 16-byte
// chunks of V elements) into a tile of row length `tp`; chunks outside the grid
// are skipped. A chunk that starts inside a row ends inside it: rows are `pitch`
// elements, a multiple of 64. Thread t takes chunks t, t + NT, ..., so the first
// warps issue most copies while the others compute. Measured at 256^3, order 4,
// FP32: 6.3e10 point-stage updates/s, against 5.7e10 when a plane's chunks are
// dealt evenly to all warps and 5.9e10 with one extra warp that issues every copy.
// Deferring the x-face points' SAT to one warp after an extra barrier per plane (as
// the 2D kernels do without a barrier of their own) measured slower here: FP32
// 5.95e10, FP64 1.29e10 against 1.32e10.
template <typename T, int NR, int NC, int V, int NT>
__device__ __forceinline__ void copy_box(T* tile, int tp, const T* src, int gj0, int gi0, int nx, int ny, int pitch,
                                         int tid) {
#pragma unroll 1
  for (int idx = tid; idx < NR * NC; idx += NT) {
    const int r = idx / NC, c = idx - r * NC;
    const int gj = gj0 + r, gi = gi0 + c * V;
    if (gj >= 0 && gj < ny && gi >= 0 && gi < nx) cp_async16(tile + r * tp + c * V, src + (gj * pitch + gi));
  }
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <typename T> struct RingExtras {
  const T* x;  // this thread's element of extra array 0; array e at x[e * stride]
  int stride;
  __device__ __forceinline__ T acc(int c) const { return x[c * stride]; }
  __device__ __forceinline__ T un(int c) const { return x[(4 + c) * stride]; }
  __device__ __forceinline__ T comp(int c) const { return x[(8 + c) * stride]; }
};

// Interior D1 over W values spaced `st` apart in shared memory, in d1_line's order.
template <typename T, int ORD>
__device__ __forceinline__ T taps_smem(const DirTaps<T>& d, const T* c, int st) {
  constexpr int W = OpShape<ORD>::W, R = (W - 1) / 2;
  T s = d.taps[0] * c[0];
#pragma unroll
  for (int q = 1; q < W; q++)
    if (q != R) s = fma(d.taps[q], c[q * st], s);
  return s;
}

template <typename T, int ORD, int STAGE>
__global__ void __launch_bounds__(kR3Threads, sizeof(T) == 8 ? SBP_R3_BLOCKS_F64 : SBP_R3_BLOCKS) wave3d_ring_kernel(const __grid_constant__ Wave3Params<T> prm) {
  using G = Ring3<T, ORD, STAGE>;
  constexpr int W = OpShape<ORD>::W, R = G::R, CS = OpShape<ORD>::CS, D = G::D;
  constexpr int TX = G::TX, TY = G::TY, PX = G::PX, SA = G::SA, SB = G::SB;
  extern __shared__ __align__(16) unsigned char w3_smem[];
  T* const sA = reinterpret_cast<T*>(w3_smem);
  T* const sB = sA + SA * G::A_SZ;
  if (prm.skip && *prm.skip) return;
  // element offsets are 32-bit: the host runs this kernel only when 4 * plane < 2^31
  const int nx = prm.nx, ny = prm.ny, nz = prm.nz;
  const int pitch = (int)prm.pitch, slab = (int)prm.slab, plane = (int)prm.plane;
  const T* __restrict__ U = prm.in;
  const T* __restrict__ V_ = U + plane;
  const T* __restrict__ Wz = V_ + plane;
  const T* __restrict__ P = Wz + plane;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
  const int i = i0 + tx, j = j0 + ty;
  const bool live = i < nx && j < ny;
  const int k0 = blockIdx.z * kR3Z;
  const int k1 = k0 + kR3Z < nz ? k0 + kR3Z : nz;
  const int col = j * pitch + i;
  constexpr int V = G::V, HX = G::HX, NT = TX * TY;
  const int tid = ty * TX + tx;
  const int pc = (ty + R) * PX + tx + HX;  // this point in a p tile
  const int uc = ty * PX + tx + HX;        // in a u tile
  const int vc = (ty + R) * TX + tx;       // in a v tile
  const int wc = ty * TX + tx;             // in a w tile / an extra array

  // group m: ring A gets plane m (if inside the grid) into slot ia, ring B plane
  // m - R (if this block's) into slot ib; the slots advance with m. The p tile is
  // copied whole (its unused corners too), the others as the stencil needs them.
  int ia = 0, ib = 0;
  auto issue = [&](int m) {
    if (m >= 0 && m < nz) {
      const int o = m * slab;
      T* a = sA + ia * G::A_SZ;
      copy_box<T, TY + 2 * R, PX / V, V, NT>(a, PX, P + o, j0 - R, i0 - HX, nx, ny, pitch, tid);
      copy_box<T, TY, TX / V, V, NT>(a + G::A_W, TX, Wz + o, j0, i0, nx, ny, pitch, tid);
    }
    ia = ia + 1 == SA ? 0 : ia + 1;
    const int kb = m - R;
    if (kb >= k0 && kb < k1) {
      const int o = kb * slab;
      T* b = sB + ib * G::B_SZ;
      copy_box<T, TY, PX / V, V, NT>(b, PX, U + o, j0, i0 - HX, nx, ny, pitch, tid);
      copy_box<T, TY + 2 * R, TX / V, V, NT>(b + G::B_V, TX, V_ + o, j0 - R, i0, nx, ny, pitch, tid);
      if constexpr (G::NEX >= 8) {
#pragma unroll
        for (int c = 0; c < 4; c++) {
          copy_box<T, TY, TX / V, V, NT>(b + G::B_X + c * TY * TX, TX, prm.acc + (c * plane + o), j0, i0, nx, ny,
                                         pitch, tid);
          copy_box<T, TY, TX / V, V, NT>(b + G::B_X + (4 + c) * TY * TX, TX, prm.un + (c * plane + o), j0, i0, nx,
                                         ny, pitch, tid);
        }
      }
      if constexpr (G::NEX == 12) {
        if (prm.compensated) {
#pragma unroll
          for (int c = 0; c < 4; c++)
            copy_box<T, TY, TX / V, V, NT>(b + G::B_X + (8 + c) * TY * TX, TX, prm.comp + (c * plane + o), j0, i0,
                                           nx, ny, pitch, tid);
        }
      }
      ib = ib + 1 == SB ? 0 : ib + 1;
    }
    cp_async_commit();
  };

#pragma unroll 1
  for (int m = k0 - R; m < k0 + R + D; m++) issue(m);
  // slots read at plane k: ring B's slot of plane k, ring A's slots of planes k - R (za) and k (ka)
  int kbs = 0, za = 0, ka = R;
  T zp[W], zw[W];  // p and w at planes k - R .. k + R of this column (register window)
#pragma unroll 1
  for (int k = k0; k < k1; k++) {
    issue(k + R + D);
    cp_async_wait<D>();  // this thread's groups up to k + R are complete
    __syncthreads();     // and every thread's
    if (live) {
      const int zn = za + 2 * R < SA ? za + 2 * R : za + 2 * R - SA;  // slot of plane k + R
      if (k == k0) {
#pragma unroll
        for (int q = 0; q < W - 1; q++) {
          const int s = za + q < SA ? za + q : za + q - SA;
          zp[q] = sA[s * G::A_SZ + pc];
          zw[q] = sA[s * G::A_SZ + G::A_W + wc];
        }
      }
      zp[W - 1] = sA[zn * G::A_SZ + pc];
      zw[W - 1] = sA[zn * G::A_SZ + G::A_W + wc];
      const T* b = sB + kbs * G::B_SZ;
      const T* a = sA + ka * G::A_SZ;  // plane k
      const int xo = k * slab + j * pitch;
      const int q = xo + i;
      T kc[4], ux, vy, wz;
      if (i >= CS && i < nx - CS) {
        kc[0] = taps_smem<T, ORD>(prm.dx, a + pc - R, 1);
        ux = taps_smem<T, ORD>(prm.dx, b + uc - R, 1);
      } else {
        kc[0] = d1_line<T, ORD>(P + xo, 1, nx, i, prm.dx);
        ux = d1_line<T, ORD>(U + xo, 1, nx, i, prm.dx);
      }
      if (j >= CS && j < ny - CS) {
        kc[1] = taps_smem<T, ORD>(prm.dy, a + pc - R * PX, PX);
        vy = taps_smem<T, ORD>(prm.dy, b + G::B_V + vc - R * TX, TX);
      } else {
        const int yo = k * slab + i;
        kc[1] = d1_line<T, ORD>(P + yo, pitch, ny, j, prm.dy);
        vy = d1_line<T, ORD>(V_ + yo, pitch, ny, j, prm.dy);
      }
      if (k >= CS && k < nz - CS) {
        kc[2] = taps_window<T, ORD>(prm.dz, zp);
        wz = taps_window<T, ORD>(prm.dz, zw);
      } else {
        kc[2] = d1_line<T, ORD>(P + col, slab, nz, k, prm.dz);
        wz = d1_line<T, ORD>(Wz + col, slab, nz, k, prm.dz);
      }
      kc[3] = ux + vy + wz;
      const T cen[4] = {b[uc], b[G::B_V + vc], zw[R], zp[R]};
      wave3d_finish<T, STAGE>(prm, i, j, k, q, kc, cen, RingExtras<T>{b + G::B_X + wc, TY * TX});
#pragma unroll
      for (int s = 0; s + 1 < W; s++) {
        zp[s] = zp[s + 1];
        zw[s] = zw[s + 1];
      }
    }
    kbs = kbs + 1 == SB ? 0 : kbs + 1;
    za = za + 1 == SA ? 0 : za + 1;
    ka = ka + 1 == SA ? 0 : ka + 1;
  }
  cp_async_wait<0>();
}

// Which form runs per precision: the plane-ring kernel for both (figures at the
// top of this file).
#ifndef SBP_W3_RING_F32
#define SBP_W3_RING_F32 1
#endif
#ifndef SBP_W3_RING_F64
#define SBP_W3_RING_F64 1
#endif
template <typename T> constexpr bool w3_ring() { return sizeof(T) == 8 ? SBP_W3_RING_F64 : SBP_W3_RING_F32; }

namespace {

// SBP_WAVE3D_COLUMN=1 in the environment selects the column kernel (read at each
// launch; the tests use it to check that form against the oracle).
inline bool w3_force_column() {
  const char* e = std::getenv("SBP_WAVE3D_COLUMN");
  return e != nullptr && e[0] == '1';
}

template <typename T, int ORD>
cudaError_t wave3d_order(int stage, const Wave3Params<T>& prm, cudaStream_t s) {
  if constexpr (w3_ring<T>()) {
    // the ring kernel's element offsets are 32-bit and its copies 16-byte aligned
    const auto al16 = [](const void* q) { return q == nullptr || ((uintptr_t)q & 15) == 0; };
    if (!w3_force_column() && 4 * prm.plane < (1LL << 31) && prm.pitch % 64 == 0 && al16(prm.in) &&
        al16(prm.acc) && al16(prm.un) && al16(prm.comp)) {
      const dim3 block(kR3X, kR3Y);
      const dim3 grid((prm.nx + kR3X - 1) / kR3X, (prm.ny + kR3Y - 1) / kR3Y, (prm.nz + kR3Z - 1) / kR3Z);
      switch (stage) {
        case ST_RHS: wave3d_ring_kernel<T, ORD, ST_RHS><<<grid, block, Ring3<T, ORD, ST_RHS>::SMEM, s>>>(prm); break;
        case ST_FIRST:
          wave3d_ring_kernel<T, ORD, ST_FIRST><<<grid, block, Ring3<T, ORD, ST_FIRST>::SMEM, s>>>(prm);
          break;
        case ST_MID: wave3d_ring_kernel<T, ORD, ST_MID><<<grid, block, Ring3<T, ORD, ST_MID>::SMEM, s>>>(prm); break;
        case ST_LAST: wave3d_ring_kernel<T, ORD, ST_LAST><<<grid, block, Ring3<T, ORD, ST_LAST>::SMEM, s>>>(prm); break;
        default: return cudaErrorInvalidValue;
      }
      return cudaGetLastError();
    }
  }
  const dim3 block(kW3X, kW3Y);
  const dim3 grid((prm.nx + kW3X - 1) / kW3X, (prm.ny + kW3Y - 1) / kW3Y, (prm.nz + kW3Z - 1) / kW3Z);
  switch (stage) {
    case ST_RHS: wave3d_stage_kernel<T, ORD, ST_RHS><<<grid, block, 0, s>>>(prm); break;
    case ST_FIRST: wave3d_stage_kernel<T, ORD, ST_FIRST><<<grid, block, 0, s>>>(prm); break;
    case ST_MID: wave3d_stage_kernel<T, ORD, ST_MID><<<grid, block, 0, s>>>(prm); break;
    case ST_LAST: wave3d_stage_kernel<T, ORD, ST_LAST><<<grid, block, 0, s>>>(prm); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace

template <typename T>
cudaError_t launch_wave3d(int order, int stage, const Wave3Params<T>& prm, cudaStream_t s) {
  if (prm.nz > 65535 * kW3Z || prm.ny > 65535 * kW3Y || prm.nz > 65535 * kR3Z || prm.ny > 65535 * kR3Y)
    return cudaErrorInvalidValue;
  switch (order) {
    case 2: return wave3d_order<T, 2>(stage, prm, s);
    case 4: return wave3d_order<T, 4>(stage, prm, s);
    case 6: return wave3d_order<T, 6>(stage, prm, s);
    default: return cudaErrorInvalidValue;
  }
}
namespace {
template <typename T, int ORD, int STAGE> cudaError_t configure_ring() {
  return cudaFuncSetAttribute(wave3d_ring_kernel<T, ORD, STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)Ring3<T, ORD, STAGE>::SMEM);
}
template <typename T, int ORD> cudaError_t configure_ring_order() {
  cudaError_t e;
  if ((e = configure_ring<T, ORD, ST_RHS>()) != cudaSuccess) return e;
  if ((e = configure_ring<T, ORD, ST_FIRST>()) != cudaSuccess) return e;
  if ((e = configure_ring<T, ORD, ST_MID>()) != cudaSuccess) return e;
  return configure_ring<T, ORD, ST_LAST>();
}
}  // namespace

template <typename T> cudaError_t configure_wave3d(int order) {
  if constexpr (!w3_ring<T>()) {
    return cudaSuccess;
  } else {
    switch (order) {
      case 2: return configure_ring_order<T, 2>();
      case 4: return configure_ring_order<T, 4>();
      case 6: return configure_ring_order<T, 6>();
      default: return cudaErrorInvalidValue;
    }
  }
}
template cudaError_t configure_wave3d<double>(int);
template cudaError_t configure_wave3d<float>(int);

template cudaError_t launch_wave3d<double>(int, int, const Wave3Params<double>&, cudaStream_t);
template cudaError_t launch_wave3d<float>(int, int, const Wave3Params<float>&, cudaStream_t);

}  // namespace sbp
