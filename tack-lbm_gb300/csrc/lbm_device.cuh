// lbm_device.cuh - device code of the D3Q19 AA-pattern stream-and-collide step.
//
// Layout in HBM: one structure-of-arrays buffer F with 19 slots of n cells,
// F[q][idx], idx = (z*ny + y)*nx + x, x fastest (the reference layout,
// lbm.py:397-402, lbm.py:426). The buffer is updated in place with the
// AA pattern: an "odd" step reads the populations arriving at a cell from its
// neighbours' slots and writes its post-collision populations into the slots
// its neighbours will read locally; an "even" step reads and writes only the
// cell's own slots (with directions swapped). Each cell touches the same
// locations it reads, so the update needs no second buffer.
//
// Storage of a population is its deviation from the lattice weight,
// delta_q = f_q - w_q, in FP16/BF16; FP32 and FP64 store f_q itself. All
// arithmetic runs on deviations (float for FP32/16/BF16, double for FP64).
//
// Boundary handling follows the reference kernel (lbm.py:410-432):
//   * halfway bounce-back from obstacle cells with the moving-wall term
//     6 w_q c_q.u_w at the link midpoint, and the momentum-exchange force;
//   * periodic x, periodic or free-slip (specular) y (PeriodicY/SlipY,
//     lbm.py:342-369), and the z analogues; a moving no-slip lid above
//     y = ny-1 for LBM_LID.
// In the AA scheme a fluid cell's post-collision population that streams
// into an obstacle cell is parked in that obstacle cell's slot, which no
// other cell reads or writes; the fluid cell picks it up (bounced) on the
// next step. Obstacle cells therefore never store anything: every reference
// step resets them to w_q (sigma = 1, lbm.py:449-456) and nothing reads their
// own values except their own bounce-back links, for which w_q is used.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include <type_traits>
#include <utility>

namespace lbmk {

// f(std::integral_constant<int, 0>{}), ..., f(std::integral_constant<int, N-1>{}):
// a loop whose index is a compile-time constant in the body.
template <typename F, int... I>
__host__ __device__ __forceinline__ void static_for_impl(F &&f, std::integer_sequence<int, I...>) {
  (f(std::integral_constant<int, I>{}), ...);
}
template <int N, typename F>
__host__ __device__ __forceinline__ void static_for(F &&f) {
  static_for_impl(f, std::make_integer_sequence<int, N>{});
}

constexpr int Q = 19;
constexpr int BX = 32;   // cells per warp along x
constexpr int BY = 4;    // rows (warps) per block
constexpr int NSUM = 8;  // r_rho, r_ux, r_uy, r_uz, r_ke, fx, fy, fz

// D3Q19 ordering of the reference (lbm.py:15-17)
__host__ __device__ constexpr int cx(int q) {
  return q == 1 || q == 7 || q == 9 || q == 11 || q == 13 ? 1
       : q == 2 || q == 8 || q == 10 || q == 12 || q == 14 ? -1 : 0;
}
__host__ __device__ constexpr int cy(int q) {
  return q == 3 || q == 7 || q == 10 || q == 15 || q == 17 ? 1
       : q == 4 || q == 8 || q == 9 || q == 16 || q == 18 ? -1 : 0;
}
__host__ __device__ constexpr int cz(int q) {
  return q == 5 || q == 11 || q == 14 || q == 15 || q == 18 ? 1
       : q == 6 || q == 12 || q == 13 || q == 16 || q == 17 ? -1 : 0;
}
// index of the direction (ex, ey, ez)
__host__ __device__ constexpr int dir(int ex, int ey, int ez) {
  int r = -1;
  for (int q = 0; q < Q; ++q)
    if (cx(q) == ex && cy(q) == ey && cz(q) == ez) r = q;
  return r;
}
__host__ __device__ constexpr int opp(int q) { return dir(-cx(q), -cy(q), -cz(q)); }

// lattice weights as the reference uploads them: float32 (lbm.py:18, lbm.py:48)
__host__ __device__ constexpr float wq(int q) {
  return q == 0 ? 1.0f / 3.0f : (q <= 6 ? 1.0f / 18.0f : 1.0f / 36.0f);
}
// sum of the float32 weights minus one (2^-26): rho = 1 + sum(delta) + W_EXCESS
constexpr double W_EXCESS = 1.4901161193847656e-08;

enum { COLL_BGK = 0, COLL_TRT = 1, COLL_LES = 2 };
enum { OBS_NONE = 0, OBS_CYL = 1, OBS_SPH = 2, OBS_BOX = 3, OBS_SINK = 4 };
enum { SIDE_PERIODIC = 0, SIDE_SLIP = 1, SIDE_LID = 2 };

struct Geo {
  int kind;
  float ox, oy, oz, r2, inv_r, hx, hy, hz;
  float r;
  // heat sink (HeatSink, lbm.py:230-276): x range [sx0, sx1), z range [sz0,
  // sz1), plate below y = sybase, fins below y = sytop every spitch cells in z
  // (sthick thick) starting at z = iz0; duct walls at y = 0 and y = ny - 1
  float sx0, sx1, sz0, sz1, sybase, sytop;
  int iz0, sthick, spitch, ny;
};

// Everything a step launch needs, passed by value (__grid_constant__).
template <typename S> struct Store;

template <typename S>
struct StepArgs {
  using P = typename Store<S>::T;  // arithmetic precision of the step
  S *slot[Q];             // slot[q] = F + q*n (slot layout)
  S *F;                   // the population buffer
  uint32_t n;             // cells (the slot stride)
  int flat;               // the step kernels address populations by 32-bit offsets from F
  int blk;                // block layout (see blocked_layout)
  uint32_t rowp;          // block layout: elements per lattice row
  int bstep[4];           // block layout, position offsets modulo 2^32: to the cell at
  int bwrap[4];           //   y - 1, y + 1, z - 1, z + 1, and across the periodic wraps
  int nx, ny, nz, nxy;
  Geo geo;
  int lateral, vertical;
  P u_lid;
  P u0, sponge_start, sponge_strength, inv_sponge_len;
  P omega_rot;
  P wall_ox, wall_oy, wall_inv_r;     // cylinder axis and 1/r for the moving-wall term
  P omega_bgk, tau0, smag_c, magic;   // smag_c = 25.456 cs^2 (lbm.py:93)
  float *fld[13];
  float4 *aux;            // temperature runs: (ux, uy, uz, tau) of every fluid cell, else null
  float2 *partials;       // NSUM compensated float pairs per block (report steps)
  int reach_lo[3], reach_hi[3];  // cells that may be solid or next to solid lie in this box
  int reach_any;                 // 0: no obstacle cell at all
  const uint32_t *masks;         // link masks of the warps in the reach box (32 words each)
  int gx, gy;             // grid dimensions in blocks (x, y)
};

// Population layouts. Slot layout: slot q of cell idx at F[q n + idx]
// (slot[q] + idx). Block layout: each lattice row is cut into 32-cell blocks
// (the last one padded) and a block keeps its 19 slots side by side, 32
// elements each, so slot q of the cell at (x, row) sits at
//   (row ceil(nx / 32) + x / 32) 19 32 + 32 q + x % 32.
// A warp (a 32-cell row segment) then finds the 19 slots of its cells at
// fixed offsets from one base, and its 19 loads fall in one 2.4 kB stretch
// of HBM (FP32; 1.2 kB in FP16/BF16). Storage types whose blocked_layout()
// holds use it wherever 32-bit offsets reach (19 x the padded cells <
// 2^32), except under the bulk-copy kernel (which streams slot rows) and
// LBM_FLAG_SLOT_POINTERS. Measured per C2 launch against the slot layout:
// FP32 0.1973 -> 0.1931 ms (report steps 0.367 -> 0.355 ms); FP16 0.1505 ->
// 0.1475 ms, but report steps 0.315 -> 0.333 ms (nine quiet steps and a
// report: 1.640 -> 1.632 ms). FP64 keeps the slot layout.
#ifndef LBM_BLOCKED_32
#define LBM_BLOCKED_32 1
#endif
#ifndef LBM_BLOCKED_16
#define LBM_BLOCKED_16 1
#endif
constexpr int BLK = 32;
__host__ __device__ constexpr bool blocked_layout(int bytes) {
  return bytes == 4 ? LBM_BLOCKED_32 != 0 : bytes == 2 ? LBM_BLOCKED_16 != 0 : false;
}

// block layout: offset of slot 0 of cell (x, row), row = z ny + y
template <typename S>
__device__ __forceinline__ uint32_t blk_pos(const StepArgs<S> &a, int row, int x) {
  return (uint32_t)row * a.rowp + (uint32_t)(x >> 5) * (uint32_t)(Q * BLK) + (uint32_t)(x & (BLK - 1));
}

// slot q of cell (x, y, z), either layout (the kernels off the per-cell fast path)
template <typename S>
__device__ __forceinline__ S *elem(const StepArgs<S> &a, int q, int x, int y, int z) {
  if (!a.blk) return a.slot[q] + ((z * a.ny + y) * a.nx + x);
  return a.F + (size_t)blk_pos(a, z * a.ny + y, x) + (size_t)(q * BLK);
}
// slot q of cell idx = (z ny + y) nx + x
template <typename S>
__device__ __forceinline__ S *elem(const StepArgs<S> &a, int q, int idx) {
  if (!a.blk) return a.slot[q] + idx;
  const int row = idx / a.nx;
  return a.F + (size_t)blk_pos(a, row, idx - row * a.nx) + (size_t)(q * BLK);
}

// Geometry of a configuration in the float32 form the kernels evaluate
// (r^2 rounded like the reference's r*r).
template <typename Cfg>
inline Geo make_geo(const Cfg &g) {
  Geo o{};
  o.kind = g.obstacle;
  o.ox = (float)g.ox;
  o.oy = (float)g.oy;
  o.oz = (float)g.oz;
  o.r = (float)g.r;
  o.r2 = (float)g.r * (float)g.r;
  o.inv_r = g.r != 0.0 ? (float)(1.0 / g.r) : 0.0f;
  o.hx = (float)g.hx;
  o.hy = (float)g.hy;
  o.hz = (float)g.hz;
  // sink = {x0, length, z0, width, base, fin_height, fin_thickness, fin_pitch}
  o.sx0 = (float)g.sink[0];
  o.sx1 = (float)(g.sink[0] + g.sink[1]);
  o.sz0 = (float)g.sink[2];
  o.sz1 = (float)(g.sink[2] + g.sink[3]);
  o.sybase = (float)(1.0 + g.sink[4]);
  o.sytop = (float)(1.0 + g.sink[4] + g.sink[5]);
  o.iz0 = (int)g.sink[2];
  o.sthick = (int)g.sink[6];
  o.spitch = g.sink[7] >= 1.0 ? (int)g.sink[7] : 1;
  o.ny = g.ny;
  return o;
}

// grid for the one-thread-per-cell utility kernels (grid-stride loops)
inline int cell_grid(long long n) {
  const long long b = (n + 255) / 256;
  return (int)(b < 152 * 32 ? b : 152 * 32);
}

// ---------------------------------------------------------------------------
// storage traits: load a deviation, store a deviation

// Population values in arithmetic: FP32 and FP64 storage keep f_q itself
// (DEV = false); FP16/BF16 storage keeps the deviation f_q - w_q (DEV = true),
// which is what the arithmetic then works on. load/store move values in that
// representation; load_value/store_value move f_q itself (host exchange),
// rounding once.
// Memory hints of the step's population traffic. In one step launch every
// location is read once and written afterwards only by the cell that read it
// (the AA scheme), and every value a cell stores depends on all of its loads
// (through the density), so:
//   * loads carry a prefetch hint (ld.global.L2::256B: the L2 fetches the
//     whole 256-byte block, which the warps of neighbouring rows and slots
//     read next);
//   * stores are streaming (st.global.cs): nothing reads them again in this
//     launch, and the next step's reads come from HBM (the populations are
//     five times the L2).
__device__ __forceinline__ float load_l2(const float *p) {
  float v;
  asm volatile("ld.global.L2::256B.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}

// the same hint for 2-byte storage (FP16/BF16: 0.8 % faster than __ldg)
__device__ __forceinline__ unsigned short load_l2_u16(const void *p) {
  unsigned short v;
  asm volatile("ld.global.L2::256B.b16 %0, [%1];" : "=h"(v) : "l"(p));
  return v;
}

template <> struct Store<float> {
  using T = float;
  static constexpr bool DEV = false;
  template <int q> __device__ static float load(const float *p) { return *p; }
  template <int q> __device__ static void store(float *p, float v) { *p = v; }
  // the same on global memory with the step's hints (any other address space faults)
  template <int q> __device__ static float gload(const float *p) { return load_l2(p); }
  template <int q> __device__ static void gstore(float *p, float v) { __stcs(p, v); }
  template <int q> __device__ static double load_value(const float *p) { return (double)*p; }
  template <int q> __device__ static void store_value(float *p, double v) { *p = (float)v; }
};
template <> struct Store<double> {
  using T = double;
  static constexpr bool DEV = false;
  template <int q> __device__ static double load(const double *p) { return *p; }
  template <int q> __device__ static void store(double *p, double v) { *p = v; }
  template <int q> __device__ static double gload(const double *p) { return *p; }
  template <int q> __device__ static void gstore(double *p, double v) { *p = v; }
  template <int q> __device__ static double load_value(const double *p) { return *p; }
  template <int q> __device__ static void store_value(double *p, double v) { *p = v; }
};
template <> struct Store<__half> {
  using T = float;
  static constexpr bool DEV = true;
  template <int q> __device__ static float load(const __half *p) { return __half2float(*p); }
  template <int q> __device__ static void store(__half *p, float d) { *p = __float2half_rn(d); }
  template <int q> __device__ static float gload(const __half *p) {
    return __half2float(__ushort_as_half(load_l2_u16(p)));
  }
  template <int q> __device__ static void gstore(__half *p, float d) { __stcs(p, __float2half_rn(d)); }
  template <int q> __device__ static double load_value(const __half *p) {
    return (double)wq(q) + (double)__half2float(*p);
  }
  template <int q> __device__ static void store_value(__half *p, double v) {
    *p = __double2half(v - (double)wq(q));
  }
};
template <> struct Store<__nv_bfloat16> {
  using T = float;
  static constexpr bool DEV = true;
  template <int q> __device__ static float load(const __nv_bfloat16 *p) { return __bfloat162float(*p); }
  template <int q> __device__ static void store(__nv_bfloat16 *p, float d) { *p = __float2bfloat16_rn(d); }
  template <int q> __device__ static float gload(const __nv_bfloat16 *p) {
    return __bfloat162float(__ushort_as_bfloat16(load_l2_u16(p)));
  }
  template <int q> __device__ static void gstore(__nv_bfloat16 *p, float d) {
    __stcs(p, __float2bfloat16_rn(d));
  }
  template <int q> __device__ static double load_value(const __nv_bfloat16 *p) {
    return (double)wq(q) + (double)__bfloat162float(*p);
  }
  template <int q> __device__ static void store_value(__nv_bfloat16 *p, double v) {
    *p = __double2bfloat16(v - (double)wq(q));
  }
};

// the value of population q at rest with rho = 1 in the representation DEV
template <typename T, bool DEV>
__host__ __device__ constexpr T rest_value(int q) {
  return DEV ? T(0) : T(wq(q));
}

// ---------------------------------------------------------------------------
// geometry: the reference's solid() tests evaluated in float32 with every
// product and sum rounded separately (no fused multiply-add), so the mask is
// reproducible on the host bit for bit (lbm.py:150-153, 177-182, 207-211).

// HeatSink.sink (lbm.py:250-261): the base plate and fins
__host__ __device__ __forceinline__ bool sink(const Geo &g, int x, int y, int z) {
  if (g.kind != OBS_SINK) return false;
  const float fx = (float)x, fy = (float)y, fz = (float)z;
  const bool inside = fx >= g.sx0 && fx < g.sx1 && fz >= g.sz0 && fz < g.sz1 && fy >= 1.0f;
  int m = (z - g.iz0) % g.spitch;
  m += m < 0 ? g.spitch : 0;
  return inside && (fy < g.sybase || (fy < g.sytop && m < g.sthick));
}

__device__ __forceinline__ bool solid(const Geo &g, int x, int y, int z) {
  if (g.kind == OBS_SINK) return y <= 0 || y >= g.ny - 1 || sink(g, x, y, z);
  const float fx = (float)x, fy = (float)y, fz = (float)z;
  if (g.kind == OBS_CYL) {
    const float dx = __fsub_rn(fx, g.ox), dy = __fsub_rn(fy, g.oy);
    return __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) < g.r2;
  }
  if (g.kind == OBS_SPH) {
    const float dx = __fsub_rn(fx, g.ox), dy = __fsub_rn(fy, g.oy), dz = __fsub_rn(fz, g.oz);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)) < g.r2;
  }
  if (g.kind == OBS_BOX) {
    const float ax = __fsub_rn(fabsf(__fsub_rn(fx, g.ox)), g.hx);
    const float ay = __fsub_rn(fabsf(__fsub_rn(fy, g.oy)), g.hy);
    const float az = __fsub_rn(fabsf(__fsub_rn(fz, g.oz)), g.hz);
    return fmaxf(fmaxf(ax, ay), az) < 0.0f;
  }
  return false;
}

// ---------------------------------------------------------------------------
// Moments, equilibrium, collisions and sponge on population values v_q
// (v = f, or v = f - w with DEV).
//
// With rho = 1 + drho and s = c_q.u, the equilibrium of lbm.py:52-55 is
//   feq_q = w_q (rho - 1.5 rho u^2 + 4.5 rho s^2 + 3 rho s);
// in the value representation the constant rho becomes rv = DEV ? drho : rho.
// The directions pair up as (q, opp q) = (2k+1, 2k+2), k = 0..8, with
// feq = w (A + B) and w (A - B) for A = rv - 1.5 rho u^2 + 4.5 rho s^2,
// B = 3 rho s. The deviation pair sums D_k = f_q + f_opp - 2 w_q and the
// differences M_k = f_q - f_opp give the density, the momentum and the
// deviation second moments S_ab = sum c_a c_b (f_q - w_q) without cancellation.
// The equilibrium's part of S_ab follows from the lattice moments of the
// weights as uploaded (float32-rounded, lbm.py:48): with W2 = sum w c_x^2 and
// W22 = sum w c_x^2 c_y^2,
//   sum c_a c_a (feq - w) = W2 (drho - 1.5 rho u^2) + 4.5 rho (W2 u_a^2 + W22 (u^2 - u_a^2)),
//   sum c_a c_b (feq - w) = 9 rho W22 u_a u_b (a != b),
// which is drho/3 + rho u_a^2 and rho u_a u_b for exact weights; subtracting it
// gives the non-equilibrium stress of lbm.py:81-91.

__host__ __device__ constexpr int pq(int k) { return 2 * k + 1; }
constexpr double W2 = 2.0 * (double)wq(1) + 8.0 * (double)wq(7);
constexpr double W22 = 4.0 * (double)wq(7);

template <typename T>
struct Moments {
  T drho, rho, ux, uy, uz;
};

// pairs k: q = 1 (1,0,0), 3 (0,1,0), 5 (0,0,1), 7 (1,1,0), 9 (1,-1,0),
//          11 (1,0,1), 13 (1,0,-1), 15 (0,1,1), 17 (0,1,-1)
template <typename T>
struct Pairs {
  T D[9], M[9];
};

template <typename T> __device__ __forceinline__ T rcp_fast(T v);
template <> __device__ __forceinline__ float rcp_fast<float>(float v) { return __fdividef(1.0f, v); }
template <> __device__ __forceinline__ double rcp_fast<double>(double v) { return 1.0 / v; }
// square root of v >= 0 (0 maps to 0)
template <typename T> __device__ __forceinline__ T sqrt_fast(T v);
template <> __device__ __forceinline__ float sqrt_fast<float>(float v) { return v * rsqrtf(fmaxf(v, 1e-37f)); }
template <> __device__ __forceinline__ double sqrt_fast<double>(double v) { return sqrt(v); }

template <typename T, bool DEV>
__device__ __forceinline__ Moments<T> moments(const T v[Q], bool fluid, Pairs<T> &pr) {
  const T off0 = DEV ? T(0) : T(wq(0));
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const T offk = DEV ? T(0) : T(2) * T(wq(pq(k)));
    pr.D[k] = (v[pq(k)] + v[pq(k) + 1]) - offk;
    pr.M[k] = v[pq(k)] - v[pq(k) + 1];
  }
  T sum = v[0] - off0;
#pragma unroll
  for (int k = 0; k < 9; ++k) sum += pr.D[k];
  Moments<T> m;
  m.drho = sum + T(W_EXCESS);
  m.rho = T(1) + m.drho;
  const T jx = pr.M[0] + pr.M[3] + pr.M[4] + pr.M[5] + pr.M[6];
  const T jy = pr.M[1] + pr.M[3] - pr.M[4] + pr.M[7] + pr.M[8];
  const T jz = pr.M[2] + pr.M[5] - pr.M[6] + pr.M[7] - pr.M[8];
  const T inv = fluid ? rcp_fast<T>(m.rho) : T(0);
  m.ux = jx * inv;
  m.uy = jy * inv;
  m.uz = jz * inv;
  return m;
}

// c_q . u of the pair's first direction q = pq(k): its first nonzero
// component is +1 and it has at most one more (no addition of a zero)
template <typename T, int k>
__device__ __forceinline__ T pair_dot(T ux, T uy, T uz) {
  constexpr int q = pq(k);
  static_assert(cx(q) == 1 || (cx(q) == 0 && (cy(q) == 1 || (cy(q) == 0 && cz(q) == 1))), "pair order");
  if constexpr (cx(q) == 1) {
    if constexpr (cy(q) != 0) return cy(q) == 1 ? ux + uy : ux - uy;
    if constexpr (cz(q) != 0) return cz(q) == 1 ? ux + uz : ux - uz;
    return ux;
  } else if constexpr (cy(q) == 1) {
    if constexpr (cz(q) != 0) return cz(q) == 1 ? uy + uz : uy - uz;
    return uy;
  } else {
    return uz;
  }
}

// A and B of every pair (see above) and the rest population's equilibrium
template <typename T, bool DEV>
__device__ __forceinline__ void eq_pairs(T rv, T rho, T ux, T uy, T uz, T A[9], T B[9], T &eq0) {
  const T base = rv - T(1.5) * rho * (ux * ux + uy * uy + uz * uz);
  const T r45 = T(4.5) * rho, r3 = T(3.0) * rho;
  eq0 = T(wq(0)) * base;
  static_for<9>([&](auto kc) {
    constexpr int k = decltype(kc)::value;
    const T sd = pair_dot<T, k>(ux, uy, uz);
    A[k] = r45 * sd * sd + base;
    B[k] = r3 * sd;
  });
}

// The equilibrium of one pair formed where it is used (the same arithmetic as
// eq_pairs), so that no array of A and B stays live across the collision.
template <typename T>
struct EqBase {
  T base, r45, r3;
};
template <typename T>
__device__ __forceinline__ EqBase<T> eq_base(T rv, T rho, T ux, T uy, T uz) {
  return EqBase<T>{rv - T(1.5) * rho * (ux * ux + uy * uy + uz * uz), T(4.5) * rho, T(3.0) * rho};
}
template <typename T, int k>
__device__ __forceinline__ void eq_pair(const EqBase<T> &e, T ux, T uy, T uz, T &A, T &B) {
  const T sd = pair_dot<T, k>(ux, uy, uz);
  A = e.r45 * sd * sd + e.base;
  B = e.r3 * sd;
}

// equilibrium values of all 19 directions
template <typename T, bool DEV>
__device__ __forceinline__ void feq_val(T rv, T rho, T ux, T uy, T uz, T eq[Q]) {
  T A[9], B[9];
  eq_pairs<T, DEV>(rv, rho, ux, uy, uz, A, B, eq[0]);
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const T w = T(wq(pq(k)));
    eq[pq(k)] = w * (A[k] + B[k]);
    eq[pq(k) + 1] = w * (A[k] - B[k]);
  }
}

template <typename T, bool DEV>
__device__ __forceinline__ T rv_of(const Moments<T> &m) {
  return DEV ? m.drho : m.rho;
}

// v <- v + om (feq - v), written v (1 - om) + om feq. With feq = w (A +- B),
// A = base + 4.5 rho s^2 and B = 3 rho s, om w feq = X +- Y for
// X = om w base + (om w 4.5 rho) s^2 and Y = (om w 3 rho) s: the three
// coefficients are formed once per weight class, then each population is
// (v keep + X) +- Y, two fused multiply-adds. (Against om w A and om w B
// formed per pair: 3.6 % faster FP16 and 1.5 % faster FP32 C2 launches.)
template <typename T>
__device__ __forceinline__ void relax_bgk(T v[Q], T om, const EqBase<T> &e, T ux, T uy, T uz) {
  const T keep = T(1) - om;
  const T om1 = om * T(wq(1)), om7 = om * T(wq(7));
  v[0] = v[0] * keep + om * (T(wq(0)) * e.base);
  const T ob1 = om1 * e.base, ob7 = om7 * e.base;
  const T o451 = om1 * e.r45, o457 = om7 * e.r45;
  const T o31 = om1 * e.r3, o37 = om7 * e.r3;
  static_for<9>([&](auto kc) {
    constexpr int k = decltype(kc)::value;
    constexpr int q = pq(k);
    const T sd = pair_dot<T, k>(ux, uy, uz);
    const T X = fma((k < 3 ? o451 : o457) * sd, sd, k < 3 ? ob1 : ob7);
    const T o3 = k < 3 ? o31 : o37;
    v[q] = fma(o3, sd, fma(v[q], keep, X));
    v[q + 1] = fma(-o3, sd, fma(v[q + 1], keep, X));
  });
}

// Relax the values v[] in place: BGK (lbm.py:60-69), TRT + Smagorinsky
// (lbm.py:96-123), LES-BGK (lbm.py:126-139).
// Returns the relaxation time (the D3Q7 temperature block's subgrid
// diffusivity uses it, lbm.py:299-301).
template <typename T, int COLL, bool DEV>
__device__ __forceinline__ T collide(T v[Q], const Moments<T> &m, const Pairs<T> &pr, T omega_bgk, T tau0,
                                     T smag_c, T magic) {
  const EqBase<T> e = eq_base<T>(rv_of<T, DEV>(m), m.rho, m.ux, m.uy, m.uz);
  if (COLL == COLL_BGK) {
    relax_bgk<T>(v, omega_bgk, e, m.ux, m.uy, m.uz);
    return tau0;
  }
  // Smagorinsky relaxation time from the non-equilibrium stress (lbm.py:72-93)
  const T uxx = m.ux * m.ux, uyy = m.uy * m.uy, uzz = m.uz * m.uz, usq = uxx + uyy + uzz;
  const T r45 = T(4.5) * m.rho;
  const T iso = T(W2) * (m.drho - T(1.5) * m.rho * usq) + r45 * T(W22) * usq;
  const T diag = r45 * T(W2 - W22);
  const T offd = T(9) * m.rho * T(W22);
  // the diagonal pair sums share the diagonal-direction pairs
  const T s34 = pr.D[3] + pr.D[4], s56 = pr.D[5] + pr.D[6], s78 = pr.D[7] + pr.D[8];
  const T pxx = ((pr.D[0] + s34) + s56) - iso - diag * uxx;
  const T pyy = ((pr.D[1] + s34) + s78) - iso - diag * uyy;
  const T pzz = ((pr.D[2] + s56) + s78) - iso - diag * uzz;
  const T pxy = (pr.D[3] - pr.D[4]) - offd * m.ux * m.uy;
  const T pxz = (pr.D[5] - pr.D[6]) - offd * m.ux * m.uz;
  const T pyz = (pr.D[7] - pr.D[8]) - offd * m.uy * m.uz;
  const T pi = sqrt_fast<T>(pxx * pxx + pyy * pyy + pzz * pzz + T(2) * (pxy * pxy + pxz * pxz + pyz * pyz));
  const T tau = T(0.5) * (tau0 + sqrt_fast<T>(tau0 * tau0 + smag_c * pi * rcp_fast<T>(m.rho)));
  if (COLL == COLL_LES) {
    relax_bgk<T>(v, rcp_fast<T>(tau), e, m.ux, m.uy, m.uz);
    return tau;
  }
  // TRT: even/odd parts relaxed at omega+ = 1/tau, omega- = 1/(magic/(tau-1/2)+1/2)
  const T hp = T(0.5) * rcp_fast<T>(tau);
  const T hm = T(0.5) * rcp_fast<T>(magic * rcp_fast<T>(tau - T(0.5)) + T(0.5));
  v[0] += T(2) * hp * (T(wq(0)) * e.base - v[0]);
  static_for<9>([&](auto kc) {
    constexpr int k = decltype(kc)::value;
    constexpr int q = pq(k);
    T A, B;
    eq_pair<T, k>(e, m.ux, m.uy, m.uz, A, B);
    const T w2 = T(2) * T(wq(q));
    // D_k - 2 w (A - rv + drho): the symmetric non-equilibrium part in deviations
    const T sym = hp * (pr.D[k] - w2 * (A - (DEV ? T(0) : T(1))));
    const T anti = hm * (pr.M[k] - w2 * B);
    v[q] = v[q] - sym - anti;
    v[q + 1] = v[q + 1] - sym + anti;
  });
  return tau;
}

// v <- feq(e1, u1) + keep (v - feq(e0, u0)), both equilibria formed pair by
// pair as they are used (no 19-value equilibrium arrays stay live).
template <typename T>
__device__ __forceinline__ void blend_eq(T v[Q], const EqBase<T> &e0, T ux0, T uy0, T uz0, const EqBase<T> &e1,
                                         T ux1, T uy1, T uz1, T keep) {
  v[0] = T(wq(0)) * e1.base + keep * (v[0] - T(wq(0)) * e0.base);
  static_for<9>([&](auto kc) {
    constexpr int k = decltype(kc)::value;
    constexpr int q = pq(k);
    const T w = T(wq(q));
    T A0, B0, A1, B1;
    eq_pair<T, k>(e0, ux0, uy0, uz0, A0, B0);
    eq_pair<T, k>(e1, ux1, uy1, uz1, A1, B1);
    v[q] = w * (A1 + B1) + keep * (v[q] - w * (A0 + B0));
    v[q + 1] = w * (A1 - B1) + keep * (v[q + 1] - w * (A0 - B0));
  });
}

// Sponge blend toward (1, u0*fluid, 0, 0) (lbm.py:446-456):
// out = feq(rho_s, u_s) + (1 - sigma)(post - feq(rho, u)), in values.
template <typename T, bool DEV>
__device__ __forceinline__ void sponge(T v[Q], const Moments<T> &m, T sigma, T u0fluid) {
  const EqBase<T> e0 = eq_base<T>(rv_of<T, DEV>(m), m.rho, m.ux, m.uy, m.uz);
  const T drho_s = m.drho - sigma * m.drho;
  const T rho_s = T(1) + drho_s;
  const T ux_s = m.ux + sigma * (u0fluid - m.ux);
  const T uy_s = (T(1) - sigma) * m.uy;
  const T uz_s = (T(1) - sigma) * m.uz;
  const EqBase<T> e1 = eq_base<T>(DEV ? drho_s : rho_s, rho_s, ux_s, uy_s, uz_s);
  blend_eq<T>(v, e0, m.ux, m.uy, m.uz, e1, ux_s, uy_s, uz_s, T(1) - sigma);
}

// ---------------------------------------------------------------------------
// Report-step sums. A float pair (Knuth's TwoSum) carries ~44 bits, so the
// warp and block sums of the float32 report fields lose nothing a float64 sum
// would keep. GB300's float64 pipe is narrow (a warp instruction costs many
// cycles whatever its active lanes), so the step kernels use no float64 at
// all: the pairs are added in float64 by the finalize kernel only.

struct CSum {
  float hi, lo;
};
__device__ __forceinline__ CSum csum_add(CSum a, CSum b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bp = __fsub_rn(s, a.hi);
  const float ap = __fsub_rn(s, bp);
  const float e = __fadd_rn(__fsub_rn(a.hi, ap), __fsub_rn(b.hi, bp));
  const float lo = __fadd_rn(__fadd_rn(a.lo, b.lo), e);
  const float hi = __fadd_rn(s, lo);
  return {hi, __fsub_rn(lo, __fsub_rn(hi, s))};
}
__device__ __forceinline__ CSum warp_csum(float v) {
  CSum x{v, 0.f};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    CSum y{__shfl_down_sync(0xffffffffu, x.hi, o), __shfl_down_sync(0xffffffffu, x.lo, o)};
    x = csum_add(x, y);
  }
  return x;
}

// Monitor sums of a report step: the 8 summed fields (r_rho, r_ux, r_uy, r_uz,
// r_ke, fx, fy, fz) are read back once by a streaming kernel, four cells per
// load when n % 4 == 0. The forces are momentum exchanged on links into
// obstacle cells, so a report step writes exact zeros for them outside the
// obstacle's reach box, and only the box is read for them (at C2 the five
// residual fields are 168 MB, the box's forces 1 MB, instead of 268 MB).
// Each thread keeps compensated float pairs over its cells, then warp and
// block pairs; every block writes 8 pairs. The last block to finish (an
// atomic ticket, no waiting) adds the blocks' pairs in float64, writes the 8
// sums and resets the ticket for the next report step.
constexpr int SUM_THREADS = 256;
constexpr int NRES = 5;  // the residual fields, summed over every cell
// Blocks per SM of field_sums_kernel: its 256 threads of ~60 registers fit 4
// per SM, so 4 per SM is one wave. With two float4 loads per field in flight
// per thread: report step 0.339 -> 0.326 ms at C2 (8 per SM, one load: two
// waves, 0.339; 4 per SM alone 0.333; two loads alone 0.336).
constexpr int SUM_BLOCKS_PER_SM = 4;

// the cells whose links may reach an obstacle cell (any = 0: none)
struct SumBox {
  int lo[3], hi[3], any, nx, ny;
};

// a + b as an exact pair (Knuth's TwoSum)
__device__ __forceinline__ CSum two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  const float ap = __fsub_rn(s, bp);
  return {s, __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp))};
}
// four values into the running pair: exact pairs of (x, y) and (z, w), their
// pair sum, then one dependent addition per load instead of four
__device__ __forceinline__ void csum4(CSum &acc, float4 v) {
  acc = csum_add(acc, csum_add(two_sum(v.x, v.y), two_sum(v.z, v.w)));
}

static __global__ void __launch_bounds__(SUM_THREADS)
field_sums_kernel(const float *const *fld, int n, SumBox box, float2 *partials, unsigned int *ticket, double *sums) {
  __shared__ CSum red[SUM_THREADS / 32][NSUM];
  __shared__ double fin[SUM_THREADS / 32][NSUM];
  __shared__ bool last;
  CSum acc[NSUM];
#pragma unroll
  for (int k = 0; k < NSUM; ++k) acc[k] = {0.f, 0.f};
  const float *f[NSUM];
#pragma unroll
  for (int k = 0; k < NSUM; ++k) f[k] = fld[5 + k];
  const int stride = (int)gridDim.x * SUM_THREADS;
  int tail = 0;
  if ((n & 3) == 0) {
    const int n4 = n >> 2;
    int i = (int)blockIdx.x * SUM_THREADS + (int)threadIdx.x;
    // two loads per field in flight before the additions
    for (; i + stride < n4; i += 2 * stride) {
      float4 v[NRES], w[NRES];
#pragma unroll
      for (int k = 0; k < NRES; ++k) {
        v[k] = __ldcs(reinterpret_cast<const float4 *>(f[k]) + i);
        w[k] = __ldcs(reinterpret_cast<const float4 *>(f[k]) + i + stride);
      }
#pragma unroll
      for (int k = 0; k < NRES; ++k) {
        csum4(acc[k], v[k]);
        csum4(acc[k], w[k]);
      }
    }
    for (; i < n4; i += stride) {
      float4 v[NRES];
#pragma unroll
      for (int k = 0; k < NRES; ++k) v[k] = reinterpret_cast<const float4 *>(f[k])[i];
#pragma unroll
      for (int k = 0; k < NRES; ++k) csum4(acc[k], v[k]);
    }
    tail = n;
  }
  for (int i = tail + (int)blockIdx.x * SUM_THREADS + (int)threadIdx.x; i < n; i += stride) {
#pragma unroll
    for (int k = 0; k < NRES; ++k) acc[k] = csum_add(acc[k], CSum{f[k][i], 0.f});
  }
  if (box.any) {
    // the forces, row by row over the reach box
    const int bx = box.hi[0] - box.lo[0] + 1, by = box.hi[1] - box.lo[1] + 1;
    const int64_t m = (int64_t)bx * by * (box.hi[2] - box.lo[2] + 1);
    for (int64_t j = (int64_t)blockIdx.x * SUM_THREADS + threadIdx.x; j < m; j += stride) {
      const int64_t r = j / bx;
      const int x = box.lo[0] + (int)(j - r * bx), y = box.lo[1] + (int)(r % by), z = box.lo[2] + (int)(r / by);
      const int idx = (z * box.ny + y) * box.nx + x;
#pragma unroll
      for (int k = NRES; k < NSUM; ++k) acc[k] = csum_add(acc[k], CSum{f[k][idx], 0.f});
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NSUM; ++k) {
    CSum x = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      CSum y{__shfl_down_sync(0xffffffffu, x.hi, o), __shfl_down_sync(0xffffffffu, x.lo, o)};
      x = csum_add(x, y);
    }
    if (lane == 0) red[warp][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < NSUM) {
    CSum s = red[0][threadIdx.x];
    for (int w = 1; w < SUM_THREADS / 32; ++w) s = csum_add(s, red[w][threadIdx.x]);
    partials[(size_t)blockIdx.x * NSUM + threadIdx.x] = make_float2(s.hi, s.lo);
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  double d[NSUM] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < (int)gridDim.x; b += SUM_THREADS) {
#pragma unroll
    for (int k = 0; k < NSUM; ++k) {
      const float2 p = __ldcg(&partials[(size_t)b * NSUM + k]);
      d[k] += (double)p.x + (double)p.y;
    }
  }
#pragma unroll
  for (int k = 0; k < NSUM; ++k) {
    double x = d[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) fin[warp][k] = x;
  }
  __syncthreads();
  if (threadIdx.x < NSUM) {
    double x = 0.0;
    for (int w = 0; w < SUM_THREADS / 32; ++w) x += fin[w][threadIdx.x];
    sums[threadIdx.x] = x;
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

// The previous report's ux, uy, uz, p of a cell. Report steps load them with
// the populations, before any store: the field and population pointers may
// alias as far as the compiler knows, so a load issued after the stores would
// add a second, unhidden memory round trip to every cell.
struct Prev {
  float ux, uy, uz, p;
};
__device__ __forceinline__ Prev load_prev(float *const fld[13], int idx) {
  return Prev{fld[0][idx], fld[1][idx], fld[2][idx], fld[3][idx]};
}

// Diagnostics of one cell (lbm.py:493-513). v[] collects the summed values
// (the bulk-copy kernel reduces them itself).
template <typename T>
__device__ __forceinline__ void diagnostics(float *const fld[13], int idx, const Moments<T> &m, float mx,
                                            float my, float mz, const Prev &o, float v[NSUM]) {
  const float rho = (float)m.rho;
  const float ux = (float)m.ux, uy = (float)m.uy, uz = (float)m.uz;
  const float p = (float)(m.drho * T(1.0 / 3.0));
  const float ke = 0.5f * rho * (ux * ux + uy * uy + uz * uz);
  const float ok = 0.5f * (o.ux * o.ux + o.uy * o.uy + o.uz * o.uz);
  const float dp = 3.0f * (p - o.p);
  const float r[5] = {dp * dp, (ux - o.ux) * (ux - o.ux), (uy - o.uy) * (uy - o.uy), (uz - o.uz) * (uz - o.uz),
                      (ke - ok) * (ke - ok)};
#pragma unroll
  for (int k = 0; k < 5; ++k) v[k] += r[k];
  v[5] += mx;
  v[6] += my;
  v[7] += mz;
  fld[0][idx] = ux;
  fld[1][idx] = uy;
  fld[2][idx] = uz;
  fld[3][idx] = p;
  fld[4][idx] = sqrtf(ux * ux + uy * uy + uz * uz);
#pragma unroll
  for (int k = 0; k < 5; ++k) fld[5 + k][idx] = r[k];
  fld[10][idx] = mx;
  fld[11][idx] = my;
  fld[12][idx] = mz;
}


// ---------------------------------------------------------------------------
// Per-cell kernel bodies. ODD selects the neighbour-reading half of the AA pair.

__device__ __forceinline__ int block_id() {
  return ((int)blockIdx.z * (int)gridDim.y + (int)blockIdx.y) * (int)gridDim.x + (int)blockIdx.x;
}


// Fast path. Offsets of the six neighbours with periodic wrap; on rows that
// touch a free-slip wall (Row) a population that would come from beyond the
// wall comes, reflected, from the row itself (lbm.py:355-369). Cells within
// reach of the obstacle carry a link mask (bit q: population q bounces back,
// MASK_SOLID: obstacle cell). A bounce-back input is read from where the cell
// parked it on the previous step: its own slot q on an odd step, the odd-step
// source location L(x, q) (inside the obstacle cell) on an even step.
template <typename S>
struct Offsets {
  int dxm, dxp, dym, dyp, dzm, dzp;
};

struct Row {
  bool ylo, yhi, zlo, zhi;  // reflections at free-slip walls below y = 0 / above y = ny-1 / z
};

constexpr uint32_t MASK_SOLID = 1u << 19;
constexpr uint32_t MASK_LINKS = MASK_SOLID - 1;

// The six neighbour offsets of a cell in its layout's element offsets: cell
// indices in the slot layout; in the block layout, positions (the x offsets
// then differ at block edges, and a row is rowp elements). Block offsets are
// formed modulo 2^32 (positions may pass 2^31), as are the sums of them.
template <bool FLAT, typename S>
__device__ __forceinline__ Offsets<S> cell_offsets(const StepArgs<S> &a, int x, int y, int z) {
  Offsets<S> o;
  if (FLAT && blocked_layout(sizeof(S))) {
    const int xm = x == 0 ? a.nx - 1 : x - 1, xq = x == a.nx - 1 ? 0 : x + 1;
    const int bx = x >> 5, lx = x & (BLK - 1);
    o.dxm = ((xm >> 5) - bx) * (Q * BLK) + ((xm & (BLK - 1)) - lx);
    o.dxp = ((xq >> 5) - bx) * (Q * BLK) + ((xq & (BLK - 1)) - lx);
    o.dym = y == 0 ? a.bwrap[0] : a.bstep[0];
    o.dyp = y == a.ny - 1 ? a.bwrap[1] : a.bstep[1];
    o.dzm = z == 0 ? a.bwrap[2] : a.bstep[2];
    o.dzp = z == a.nz - 1 ? a.bwrap[3] : a.bstep[3];
    return o;
  }
  o.dxm = x == 0 ? a.nx - 1 : -1;
  o.dxp = x == a.nx - 1 ? 1 - a.nx : 1;
  o.dym = y == 0 ? (a.ny - 1) * a.nx : -a.nx;
  o.dyp = y == a.ny - 1 ? -(a.ny - 1) * a.nx : a.nx;
  o.dzm = z == 0 ? (a.nz - 1) * a.nxy : -a.nxy;
  o.dzp = z == a.nz - 1 ? -(a.nz - 1) * a.nxy : a.nxy;
  return o;
}

// An odd step stores each population where it read one (src_loc), so the 19
// load addresses could simply be kept for the stores: 19 pointers live across
// the whole collision. opaque_store<S>() forms the store addresses again from
// copies of the cell index and offsets the compiler cannot identify with the
// originals, which keeps 7 integers live instead. That frees the registers
// for more blocks per SM (step_min_blocks). In slot rows it made 8 blocks the
// best count (the 2-byte kernels: 7 blocks 3 % slower with it, 8 blocks 6 %
// faster than 7 without it); in 32-cell blocks FP16 runs 0.146 ms per C2
// launch with it and 0.164 without (8 blocks). FP64 does not use it.
#ifndef LBM_OPAQUE_STORE_16
#define LBM_OPAQUE_STORE_16 1
#endif
#ifndef LBM_OPAQUE_STORE_32
#define LBM_OPAQUE_STORE_32 1
#endif
template <typename S>
__host__ __device__ constexpr bool opaque_store() {
  return sizeof(S) == 2 ? LBM_OPAQUE_STORE_16 != 0 : sizeof(S) == 4 && LBM_OPAQUE_STORE_32 != 0;
}

// a copy of v the compiler cannot see through (no common subexpression with v)
__device__ __forceinline__ int opaque(int v) {
  int r;
  asm volatile("mov.b32 %0, %1;" : "=r"(r) : "r"(v));
  return r;
}
template <typename S>
__device__ __forceinline__ Offsets<S> opaque(const Offsets<S> &o) {
  return Offsets<S>{opaque(o.dxm), opaque(o.dxp), opaque(o.dym), opaque(o.dyp), opaque(o.dzm), opaque(o.dzp)};
}

template <typename S>
__device__ __forceinline__ Row row_of(const StepArgs<S> &a, int y, int z) {
  Row r;
  r.ylo = a.lateral != SIDE_PERIODIC && y == 0;
  r.yhi = a.lateral == SIDE_SLIP && y == a.ny - 1;
  r.zlo = a.vertical != SIDE_PERIODIC && z == 0;
  r.zhi = a.vertical != SIDE_PERIODIC && z == a.nz - 1;
  return r;
}

// Slot q at element offset e (a cell index, or a block position). FLAT
// (lattices whose offsets fit 32 bits, which the step kernels check once per
// launch) forms it from the one base pointer F: in the slot layout from the
// 32-bit offset q n + e (two instructions, where the 19 slot pointers of the
// other form each have to be fetched from the kernel's parameter bank again:
// 3-7 % faster per C2 launch in FP32 and FP16); in the block layout q 32 is
// a constant offset of the load or store itself.
template <bool FLAT, typename S>
__device__ __forceinline__ S *slot_at(const StepArgs<S> &a, int q, uint32_t e) {
  if (FLAT && blocked_layout(sizeof(S))) return a.F + (size_t)e + q * BLK;
  if (FLAT) return a.F + (size_t)((uint32_t)q * a.n + e);
  return a.slot[q] + (int)e;
}

// L(x, q): where population q of the cell streams from (odd steps read it there)
template <int q, bool SPECIAL, bool FLAT, typename S>
__device__ __forceinline__ S *src_loc(const StepArgs<S> &a, uint32_t idx, const Offsets<S> &o, const Row &r) {
  const int xp = cx(q) == 1 ? o.dxm : cx(q) == -1 ? o.dxp : 0;
  const int yp = cy(q) == 1 ? o.dym : cy(q) == -1 ? o.dyp : 0;
  const int zp = cz(q) == 1 ? o.dzm : cz(q) == -1 ? o.dzp : 0;
  if (!SPECIAL) return slot_at<FLAT>(a, opp(q), idx + (uint32_t)xp + (uint32_t)yp + (uint32_t)zp);
  const bool ry = (cy(q) == 1 && r.ylo) || (cy(q) == -1 && r.yhi);
  const bool rz = (cz(q) == 1 && r.zlo) || (cz(q) == -1 && r.zhi);
  constexpr int s00 = opp(q);
  constexpr int s01 = opp(dir(cx(q), cy(q), -cz(q)));
  constexpr int s10 = opp(dir(cx(q), -cy(q), cz(q)));
  constexpr int s11 = opp(dir(cx(q), -cy(q), -cz(q)));
  const int slot = ry ? (rz ? s11 : s10) : (rz ? s01 : s00);
  return slot_at<FLAT>(a, slot, idx + (uint32_t)xp + (uint32_t)(ry ? 0 : yp) + (uint32_t)(rz ? 0 : zp));
}

// moving-wall term 6 w_q c_q.u_w of a bounce link at its midpoint (lbm.py:417-428)
template <int q, typename S>
__device__ __forceinline__ typename Store<S>::T wall_term(const StepArgs<S> &a, int x, int y) {
  using T = typename Store<S>::T;
  if (a.geo.kind != OBS_CYL) return T(0);
  const T xm = T(x) - T(0.5) * T(cx(q));
  const T ym = T(y) - T(0.5) * T(cy(q));
  const T vx = a.omega_rot * (-(ym - a.wall_oy) * a.wall_inv_r);
  const T vy = a.omega_rot * ((xm - a.wall_ox) * a.wall_inv_r);
  return T(6) * T(wq(q)) * (T(cx(q)) * vx + T(cy(q)) * vy);
}

template <typename S, bool ODD, bool SPECIAL, bool FLAT>
__device__ __forceinline__ void fast_load(const StepArgs<S> &a, uint32_t ip, const Offsets<S> &o, const Row &r,
                                          uint32_t m, typename Store<S>::T d[Q]) {
  // (report steps load the previous fields beside this, see load_prev)
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    S *own = slot_at<FLAT>(a, q, ip);
    const S *addr;
    if (!SPECIAL) {
      addr = ODD ? src_loc<q, false, FLAT>(a, ip, o, r) : own;
    } else {
      const bool b = (m >> q) & 1u;
      S *src = src_loc<q, true, FLAT>(a, ip, o, r);
      addr = ODD ? (b ? own : src) : (b ? src : own);
    }
    d[q] = Store<S>::template gload<q>(addr);
  });
}

// Moments, collision, temperature coupling and sponge of a fluid cell (x, idx)
// with inputs d[]; d[] becomes the post-collision populations.
template <typename S, int COLL>
__device__ __forceinline__ Moments<typename Store<S>::T> fluid_update(const StepArgs<S> &a, int x, int idx,
                                                                     typename Store<S>::T d[Q]) {
  using T = typename Store<S>::T;
  constexpr bool DEV = Store<S>::DEV;
  Pairs<T> pr;
  const Moments<T> mo = moments<T, DEV>(d, true, pr);
  const T tau = collide<T, COLL, DEV>(d, mo, pr, a.omega_bgk, a.tau0, a.smag_c, a.magic);
  // the temperature coupling (FP32 storage only)
  if (sizeof(S) == 4 && a.aux) a.aux[idx] = make_float4((float)mo.ux, (float)mo.uy, (float)mo.uz, (float)tau);
  const T t = fmax(T(0), (T(x) - a.sponge_start) * a.inv_sponge_len);
  const T sigma = a.sponge_strength * t * t;
  if (sigma != T(0)) sponge<T, DEV>(d, mo, sigma, a.u0);
  return mo;
}

// The rest of the cell's step after fast_load: bounce-back links, the update,
// the stores and the report fields. idx indexes the fields, ip the populations.
template <typename S, int COLL, bool REPORT, bool ODD, bool SPECIAL, bool FLAT>
__device__ __forceinline__ void fast_finish(const StepArgs<S> &a, int x, int y, int idx, uint32_t ip,
                                            const Offsets<S> &o,
                                            const Row &r, uint32_t m, typename Store<S>::T d[Q], const Prev &prev,
                                            float v[NSUM]) {
  using T = typename Store<S>::T;
  constexpr bool DEV = Store<S>::DEV;
  const bool here = SPECIAL && (m & MASK_SOLID);
  float mx = 0.f, my = 0.f, mz = 0.f;
  if (SPECIAL && (m & MASK_LINKS)) {
    // bounce-back links (lbm.py:426-432): the value read is the cell's own
    // population coming back, plus the moving-wall term
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      if ((m >> q) & 1u) {
        const T wt = wall_term<q>(a, x, y);
        if (here) {
          d[q] = rest_value<T, DEV>(q) + wt;
        } else {
          const T got = d[q];
          d[q] = got + wt;
          const float hit = (float)(T(2) * (got + (DEV ? T(wq(q)) : T(0))) + wt);
          mx += hit * (float)(-cx(q));
          my += hit * (float)(-cy(q));
          mz += hit * (float)(-cz(q));
        }
      }
    });
  }
  Moments<T> mo;
  if (!here) {
    mo = fluid_update<S, COLL>(a, x, idx, d);
    const uint32_t ip_s = opaque_store<S>() ? (uint32_t)opaque((int)ip) : ip;
    const Offsets<S> o_s = opaque_store<S>() ? opaque(o) : o;
    static_for<Q>([&](auto pc) {
      constexpr int p = decltype(pc)::value;
      // population p moves to x + c_p: the odd-step source location of direction opp(p)
      if (ODD) Store<S>::template gstore<p>(src_loc<opp(p), SPECIAL, FLAT>(a, ip_s, o_s, r), d[p]);
      else Store<S>::template gstore<p>(slot_at<FLAT>(a, opp(p), ip), d[p]);
    });
  } else {
    Pairs<T> pr;
    mo = moments<T, DEV>(d, false, pr);
  }
  if (REPORT) diagnostics<T>(a.fld, idx, mo, mx, my, mz, prev, v);
}

template <typename S>
struct Link {
  S *L;        // where population q of this cell is read from on an odd step
  bool lid;    // the link crosses the moving lid
  bool wall;   // the source cell is an obstacle cell
  typename Store<S>::T cu;  // c_q . u_wall (bounce links only)
};

// geo = false skips the obstacle test (a cell with no obstacle cell within reach)
template <typename S, int q>
__device__ __forceinline__ Link<S> make_link(const StepArgs<S> &a, int x, int y, int z, bool geo = true) {
  using T = typename Store<S>::T;
  Link<S> k;
  int xs = x - cx(q);
  xs += xs < 0 ? a.nx : 0;
  xs -= xs >= a.nx ? a.nx : 0;
  int ys = y - cy(q), zs = z - cz(q);
  bool ry = false, rz = false;  // the source population is mirrored in y / z
  k.lid = false;
  if (a.lateral == SIDE_PERIODIC) {
    ys += ys < 0 ? a.ny : 0;
    ys -= ys >= a.ny ? a.ny : 0;
  } else {
    const bool lo = ys < 0, hi = ys >= a.ny;
    k.lid = hi && a.lateral == SIDE_LID;
    ry = lo || (hi && a.lateral == SIDE_SLIP);
    ys = (ry || k.lid) ? y : ys;
  }
  if (a.vertical == SIDE_PERIODIC) {
    zs += zs < 0 ? a.nz : 0;
    zs -= zs >= a.nz ? a.nz : 0;
  } else {
    rz = zs < 0 || zs >= a.nz;
    zs = rz ? z : zs;
  }
  k.wall = geo && !k.lid && solid(a.geo, xs, ys, zs);
  // the source population (cx, +-cy, +-cz) sits, in the even view, in the slot of its opposite
  constexpr int s00 = opp(q);
  constexpr int s01 = opp(dir(cx(q), cy(q), -cz(q)));
  constexpr int s10 = opp(dir(cx(q), -cy(q), cz(q)));
  constexpr int s11 = opp(dir(cx(q), -cy(q), -cz(q)));
  k.L = elem(a, ry ? (rz ? s11 : s10) : (rz ? s01 : s00), xs, ys, zs);
  // moving-wall term at the link midpoint (lbm.py:417-425)
  T cu = T(0);
  if (k.lid) {
    cu = T(cx(q)) * a.u_lid;
  } else if (a.geo.kind == OBS_CYL) {
    const T xm = T(x) - T(0.5) * T(cx(q));
    const T ym = T(y) - T(0.5) * T(cy(q));
    const T vx = a.omega_rot * (-(ym - a.wall_oy) * a.wall_inv_r);
    const T vy = a.omega_rot * ((xm - a.wall_ox) * a.wall_inv_r);
    cu = T(cx(q)) * vx + T(cy(q)) * vy;
  }
  k.cu = cu;
  return k;
}

// General path: the links of a cell evaluated one by one (lbm.py:410-432):
// walls, reflections, the lid, and - when geo - the obstacle.
template <typename S, int COLL, bool REPORT, bool ODD>
__device__ __forceinline__ void general_cell(const StepArgs<S> &a, int x, int y, int z, int idx, bool geo,
                                             float v[NSUM]) {
  using T = typename Store<S>::T;
  constexpr bool DEV = Store<S>::DEV;
  const bool here = geo && solid(a.geo, x, y, z);
  if (here && !REPORT) return;
  Prev prev{0.f, 0.f, 0.f, 0.f};
  if (REPORT) prev = load_prev(a.fld, idx);
  T d[Q];
  float mx = 0.f, my = 0.f, mz = 0.f;
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    const Link<S> k = make_link<S, q>(a, x, y, z, geo);
    const bool bb = k.lid || k.wall;
    const T wall_term = T(6) * T(wq(q)) * k.cu;
    T val;
    if (here) {
      // obstacle cell: streamed-in values, or its own w_q on its bounce links
      if (bb) val = rest_value<T, DEV>(q) + wall_term;
      else val = ODD ? Store<S>::template gload<q>(k.L) : Store<S>::template gload<q>(elem(a, q, x, y, z));
    } else {
      S *src;
      if (ODD) src = bb ? elem(a, q, x, y, z) : k.L;
      else src = k.wall ? k.L : elem(a, q, x, y, z);
      const T got = Store<S>::template gload<q>(src);
      val = bb ? got + wall_term : got;
      if (k.wall) {
        // momentum exchange (lbm.py:429-432); bounced = the population just read
        const float hit = (float)(T(2) * (got + (DEV ? T(wq(q)) : T(0))) + wall_term);
        mx += hit * (float)(-cx(q));
        my += hit * (float)(-cy(q));
        mz += hit * (float)(-cz(q));
      }
    }
    d[q] = val;
  });
  Pairs<T> pr;
  const Moments<T> m = moments<T, DEV>(d, !here, pr);
  if (!here) {
    const T tau = collide<T, COLL, DEV>(d, m, pr, a.omega_bgk, a.tau0, a.smag_c, a.magic);
    if (a.aux) a.aux[idx] = make_float4((float)m.ux, (float)m.uy, (float)m.uz, (float)tau);
    const T t = fmax(T(0), (T(x) - a.sponge_start) * a.inv_sponge_len);
    const T sigma = a.sponge_strength * t * t;
    if (sigma != T(0)) sponge<T, DEV>(d, m, sigma, a.u0);
    static_for<Q>([&](auto pc) {
      constexpr int p = decltype(pc)::value;
      constexpr int o = opp(p);
      S *dst;
      if (ODD) {
        const Link<S> k = make_link<S, o>(a, x, y, z, geo);
        dst = k.lid ? elem(a, o, x, y, z) : k.L;
      } else {
        dst = elem(a, o, x, y, z);
      }
      Store<S>::template gstore<p>(dst, d[p]);
    });
  }
  if (REPORT) diagnostics<T>(a.fld, idx, m, mx, my, mz, prev, v);
}

// A warp is one row segment of 32 cells, so every choice below is uniform per warp.

// Is the warp [x0, x0+32) x {y} x {z} inside the obstacle's reach box?
// Returns its first link-mask word, or -1.
template <typename S>
__device__ __forceinline__ int mask_slot(const StepArgs<S> &a, int x0, int y, int z) {
  if (!a.reach_any || x0 + BX - 1 < a.reach_lo[0] || x0 > a.reach_hi[0] || y < a.reach_lo[1] ||
      y > a.reach_hi[1] || z < a.reach_lo[2] || z > a.reach_hi[2])
    return -1;
  const int w0 = a.reach_lo[0] / BX, nw = a.reach_hi[0] / BX - w0 + 1;
  const int nyr = a.reach_hi[1] - a.reach_lo[1] + 1;
  return (((z - a.reach_lo[2]) * nyr + (y - a.reach_lo[1])) * nw + (x0 / BX - w0)) * BX;
}

// The lid row (the top row under LBM_LID) is left to general_kernel.
template <typename S>
__device__ __forceinline__ bool lid_row(const StepArgs<S> &a, int y) {
  return a.lateral == SIDE_LID && y == a.ny - 1;
}

// Resident step_kernel blocks per SM, by storage width, for quiet and report
// steps. Fewer registers per thread buy resident warps (more loads in
// flight); the odd step's store addresses are formed again (opaque_store)
// so that the 19 load addresses need not stay live. Measured per C2 launch
// (event-timed, 32-cell block layout): FP32 quiet 9 blocks (56 registers)
// 0.1918 ms against 0.1932 at 8 (64 registers; in slot rows 8 blocks beat 7,
// 6 and 5: 0.203, 0.206, 0.223-0.230, 0.225); FP32 report steps 0.355 ms at
// 8 against 0.380 at 9. FP16/BF16 quiet 9 blocks 0.1390 ms against 0.1460
// at 8 and 0.1639 at 10 (48 registers, heavy spills); FP16 report steps
// 0.334 ms at 8 against 0.341 at 9. FP64 (the oracle-precision runs, twice
// the registers per value) keeps 5.
#ifndef LBM_STEP_MIN_BLOCKS
#define LBM_STEP_MIN_BLOCKS 9
#endif
#ifndef LBM_STEP_MIN_BLOCKS_16
#define LBM_STEP_MIN_BLOCKS_16 9
#endif
#ifndef LBM_STEP_MIN_BLOCKS_64
#define LBM_STEP_MIN_BLOCKS_64 5
#endif
#ifndef LBM_STEP_MIN_BLOCKS_REPORT
#define LBM_STEP_MIN_BLOCKS_REPORT 8
#endif
#ifndef LBM_STEP_MIN_BLOCKS_REPORT_16
#define LBM_STEP_MIN_BLOCKS_REPORT_16 8
#endif
template <typename S, bool REPORT = false>
__host__ __device__ constexpr int step_min_blocks() {
  return sizeof(S) == 8   ? LBM_STEP_MIN_BLOCKS_64
         : sizeof(S) == 2 ? (REPORT ? LBM_STEP_MIN_BLOCKS_REPORT_16 : LBM_STEP_MIN_BLOCKS_16)
                          : (REPORT ? LBM_STEP_MIN_BLOCKS_REPORT : LBM_STEP_MIN_BLOCKS);
}

// One cell of the per-cell kernels: the warp is the 32-cell row segment at x0.
template <typename S, int COLL, bool REPORT, bool ODD, bool FLAT>
__device__ __forceinline__ void cell_step(const StepArgs<S> &a, int x0, int x, int y, int z) {
  using T = typename Store<S>::T;
  float v[NSUM] = {0, 0, 0, 0, 0, 0, 0, 0};
  // a warp in the obstacle's reach box whose 32 link masks are all zero (no
  // solid cell, no solid neighbour) takes the unmasked path; every lane
  // votes, including those past the lattice's end (their mask words are 0)
  const int ms = mask_slot(a, x0, y, z);
  const uint32_t m = ms >= 0 ? a.masks[ms + (int)threadIdx.x] : 0u;
  const bool walls = ms >= 0 && __any_sync(0xffffffffu, m != 0u);
  if (y < a.ny && !lid_row(a, y) && x < a.nx) {
    const int idx = (z * a.ny + y) * a.nx + x;
    const Row r = row_of(a, y, z);
    const Offsets<S> o = cell_offsets<FLAT>(a, x, y, z);
    const uint32_t ip = FLAT && blocked_layout(sizeof(S)) ? blk_pos(a, z * a.ny + y, x) : (uint32_t)idx;
    T d[Q];
    Prev prev{0.f, 0.f, 0.f, 0.f};
    if (!(r.ylo || r.yhi || r.zlo || r.zhi) && !walls) {
      if (REPORT) prev = load_prev(a.fld, idx);
      fast_load<S, ODD, false, FLAT>(a, ip, o, r, 0u, d);
      fast_finish<S, COLL, REPORT, ODD, false, FLAT>(a, x, y, idx, ip, o, r, 0u, d, prev, v);
    } else {
      if (REPORT || !(m & MASK_SOLID)) {
        if (REPORT) prev = load_prev(a.fld, idx);
        fast_load<S, ODD, true, FLAT>(a, ip, o, r, m, d);
        fast_finish<S, COLL, REPORT, ODD, true, FLAT>(a, x, y, idx, ip, o, r, m, d, prev, v);
      }
    }
  }
}

// Warps of a step_kernel block along x: 2 for 4-byte storage (a 64 x 2-cell
// tile, 2 % faster than 32 x 4 in FP32), 1 otherwise (32 x 4 cells).
#ifndef LBM_TILE_WARPS_X_32
#define LBM_TILE_WARPS_X_32 2
#endif
#ifndef LBM_TILE_WARPS_X_16
#define LBM_TILE_WARPS_X_16 1
#endif
template <typename S>
__host__ __device__ constexpr int tile_warps_x() {
  return sizeof(S) == 4 ? LBM_TILE_WARPS_X_32 : sizeof(S) == 2 ? LBM_TILE_WARPS_X_16 : 1;
}

template <typename S, int COLL, bool REPORT, bool ODD>
__global__ void __launch_bounds__(BX * BY, (step_min_blocks<S, REPORT>()))
step_kernel(const __grid_constant__ StepArgs<S> a) {
  constexpr int TX = tile_warps_x<S>(), TY = BY / TX;
  const int wx = (int)threadIdx.y % TX, wy = (int)threadIdx.y / TX;
  const int x0 = ((int)blockIdx.x * TX + wx) * BX;
  const int x = x0 + (int)threadIdx.x, y = (int)blockIdx.y * TY + wy, z = (int)blockIdx.z;
  if (a.flat) cell_step<S, COLL, REPORT, ODD, true>(a, x0, x, y, z);
  else cell_step<S, COLL, REPORT, ODD, false>(a, x0, x, y, z);
}

// Link masks of the warps within the obstacle's reach, one warp per 32 cells.
template <typename S>
__global__ void warp_mask_kernel(const __grid_constant__ StepArgs<S> a, uint32_t *masks) {
  const int x0 = (int)blockIdx.x * BX;
  const int y = (int)blockIdx.y, z = (int)blockIdx.z;
  const int ms = mask_slot(a, x0, y, z);
  if (ms < 0) return;
  const int x = x0 + (int)threadIdx.x;
  uint32_t m = 0;
  if (x < a.nx) {
    if (solid(a.geo, x, y, z)) m |= MASK_SOLID;
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      if (make_link<S, q>(a, x, y, z).wall) m |= 1u << q;
    });
  }
  masks[ms + (int)threadIdx.x] = m;
}

// General kernel: the special warps, four per block, from a list of
// (z*ny + y)*wx + x0/32 row-segment ids. Report sums go to the partial rows
// after the fast kernel's.
template <typename S, int COLL, bool REPORT, bool ODD>
__global__ void __launch_bounds__(BX * BY)
general_kernel(const __grid_constant__ StepArgs<S> a, const int *list, int count, int wx, int row0) {
  const int k = (int)blockIdx.x * BY + (int)threadIdx.y;
  float v[NSUM] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (k < count) {
    const int id = list[k];
    const int x0 = (id % wx) * BX;
    const int row = id / wx;
    const int y = row % a.ny, z = row / a.ny;
    const int x = x0 + (int)threadIdx.x;
    if (x < a.nx)
      general_cell<S, COLL, REPORT, ODD>(a, x, y, z, (z * a.ny + y) * a.nx + x, mask_slot(a, x0, y, z) >= 0, v);
  }
  (void)row0;
}

// ---------------------------------------------------------------------------
// Population exchange in the reference layout f[q*n + idx] and initial states.

__device__ __forceinline__ void decode(int idx, int nx, int ny, int &x, int &y, int &z) {
  x = idx % nx;
  y = (idx / nx) % ny;
  z = idx / (nx * ny);
}

template <typename S, typename V>
__global__ void import_kernel(const __grid_constant__ StepArgs<S> a, const V *src, int n) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    // even view: population q of cell idx sits in slot opp(q)
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      Store<S>::template store_value<q>(elem(a, opp(q), idx), (double)src[(size_t)q * n + idx]);
    });
  }
}

// odd_next = 1: even view (slot opp(q) of the cell); 0: odd view (where the
// last odd step put population q). Obstacle cells read back as w_q.
template <typename S, typename V>
__global__ void export_kernel(const __grid_constant__ StepArgs<S> a, V *dst, int n, int odd_next) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    int x, y, z;
    decode(idx, a.nx, a.ny, x, y, z);
    const bool here = solid(a.geo, x, y, z);
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      constexpr int o = opp(q);
      double v;
      if (here) {
        v = (double)wq(q);
      } else if (odd_next) {
        v = Store<S>::template load_value<q>(elem(a, o, x, y, z));
      } else {
        const Link<S> k = make_link<S, o>(a, x, y, z);
        v = Store<S>::template load_value<q>(k.lid ? elem(a, o, x, y, z) : k.L);
      }
      dst[(size_t)q * n + idx] = (V)v;
    });
  }
}

// lbm_init (lbm.py:383-394), written in the even view
template <typename S>
__global__ void init_kernel(const __grid_constant__ StepArgs<S> a, float seed_amp, int n) {
  using T = typename Store<S>::T;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    int x, y, z;
    decode(idx, a.nx, a.ny, x, y, z);
    const T fluid = solid(a.geo, x, y, z) ? T(0) : T(1);
    const T ux = a.u0 * fluid;
    const float ang_x = 6.2831853f * (float)x / (float)a.nx;
    const float ang_z = 6.2831853f * (float)z / (float)a.nz;
    const T uy = T(seed_amp) * a.u0 * fluid * T(sinf(ang_x)) * T(cosf(ang_z));
    T eq[Q];
    feq_val<T, Store<S>::DEV>(Store<S>::DEV ? T(0) : T(1), T(1), ux, uy, T(0), eq);
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      Store<S>::template store<q>(elem(a, opp(q), x, y, z), eq[q]);
    });
  }
}

// splitmix64 (Steele, Lea, Flood 2014; constants as published by Vigna)
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
// uniform in (0, 1) from draw k of cell idx: 24 random bits, centred
__host__ __device__ __forceinline__ float uniform01(uint64_t key, uint64_t idx, int k) {
  const uint64_t h = splitmix64(key + idx * 8ull + (uint64_t)k);
  return ((float)(uint32_t)(h >> 40) + 0.5f) * 5.9604644775390625e-08f;  // 2^-24
}

// Equilibrium with rho = 1 + rho_sigma N(0,1) and u = (u0,0,0) + U(-a,a)^3 in fluid cells.
template <typename S>
__global__ void init_random_kernel(const __grid_constant__ StepArgs<S> a, float rho_sigma,
                                   float u_noise, uint64_t key, int n) {
  using T = typename Store<S>::T;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    int x, y, z;
    decode(idx, a.nx, a.ny, x, y, z);
    T drho = T(0), ux = T(0), uy = T(0), uz = T(0);
    if (!solid(a.geo, x, y, z)) {
      const float u1 = uniform01(key, (uint64_t)idx, 0), u2 = uniform01(key, (uint64_t)idx, 1);
      const float g = sqrtf(-2.0f * logf(u1)) * cosf(6.28318530717958647692f * u2);
      drho = T(rho_sigma * g);
      ux = a.u0 + T(u_noise * (2.0f * uniform01(key, (uint64_t)idx, 2) - 1.0f));
      uy = T(u_noise * (2.0f * uniform01(key, (uint64_t)idx, 3) - 1.0f));
      uz = T(u_noise * (2.0f * uniform01(key, (uint64_t)idx, 4) - 1.0f));
    }
    T eq[Q];
    feq_val<T, Store<S>::DEV>(Store<S>::DEV ? drho : T(1) + drho, T(1) + drho, ux, uy, uz, eq);
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      Store<S>::template store<q>(elem(a, opp(q), x, y, z), eq[q]);
    });
  }
}

}  // namespace lbmk
