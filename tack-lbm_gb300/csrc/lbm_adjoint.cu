// lbm_adjoint.cu - gradients of time-averaged drag through the LES step: a
// differentiable form of the step, its hand-written adjoint kernel, and the
// checkpoint/recompute driver behind the lbm_adj_* entry points.
//
// Differentiable model (no reference counterpart; it reduces to the
// reference step of lbm.py:397-456 when phi is 0/1). The cylinder along z is a
// smoothed solid fraction
//     phi(x) = (1 + tanh((r - d(x)) / width)) / 2,  d = distance to the axis (ox, oy),
// which replaces the binary solid() test in every place the reference uses it:
//   * streaming with halfway bounce-back (lbm.py:426-428): for direction q the
//     pulled value p = f[q](x - c_q) and the bounced value b = f[opp q](x) give
//         g_q = p + phi(x - c_q) (b - p);
//   * the momentum-exchange force (lbm.py:429-432) with fluid = 1 - phi(x):
//         F = sum_q phi(x - c_q) fluid 2 b c_opp(q);
//   * u = fluid j / rho (lbm.py:437-439);
//   * the sponge blend (lbm.py:446-456) with sigma = 1 - fluid (1 - S t^2),
//     which is max(here, S t^2) for a 0/1 solid.
// The collision is LES-BGK with the Smagorinsky relaxation time of
// lbm.py:72-93 and 126-139, every boundary is periodic, there is no rotation,
// and the start state is lbm_init (lbm.py:383-394).
//
// Representation. The states are kept as deviations d_q = f_q - w_q from the
// float32 lattice weights (the weights the reference uploads, lbm.py:48), in
// T = float or double, on A/B buffers d[q*n + idx]; the arithmetic is the
// production step's (lbm_device.cuh): the density from deviation pair sums,
// the equilibrium as w_q (drho + rho (3 s + 4.5 s^2 - 1.5 u^2)) and the
// non-equilibrium stress as pair sums minus the equilibrium's analytic second
// moments. This is the same function of f as the plain form, but no quantity
// of size w_q is ever subtracted from another: in float32 the stress |Pi|
// (about 1e-5 here) keeps its digits, where the plain form loses them to the
// rounding of f itself (4e-9 per value).
//
// Loss: L = 1/(N_l * 0.5 U^2 D nz) * sum over steps t = loss_start..steps of
// F_x(t), F_x(t) the x force that step t computes from f_{t-1}.
// Parameters: U (inflow / sponge target and start state), tau0 (= 3 nu + 1/2),
// Cs and the radius r.
//
// Reverse sweep. With lambda_t = dL/df_t, step t's cell x reads the adjoint of
// its outputs lambda_t[q](x), recomputes its own forward arithmetic from
// f_{t-1}, and applies the transposed Jacobians of the sponge blend, the
// relaxation, the Smagorinsky time, the equilibria, the moments and the
// bounce-back blend. What lands on f_{t-1}[opp q](x) (the bounced value, the
// cell's own slot) goes to B[opp q](x); what lands on the pulled value
// f_{t-1}[q](x - c_q) goes to G[q](x) at the pulling cell. The next reverse
// step assembles lambda_{t-1}[q](x) = B[q](x) + G[q](x + c_q): the streaming
// transpose is a gather inside the next kernel, so one reverse step is one
// launch. Checkpoints of f every K steps are kept by the forward run; the
// reverse sweep recomputes each segment's states from its checkpoint.
//
// The obstacle band. phi is exactly zero (in T) beyond a few widths from the
// surface. A 32 x 4 x 1 block none of whose cells or their 18 sources has
// phi != 0 is outside the band: there g_q = p, fluid = 1, nothing bounces, no
// force is taken and B is never touched (its entries there are zero). Such
// blocks - most of the lattice - move 152 B per cell forward (the pull and
// the store) and 228 B per cell in reverse (the pull, the G gather, the G
// store); band blocks also read phi and the bounced values and write B.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "lbm_device.cuh"
#include "lbm_host.h"

namespace lbma {

using namespace lbmk;

constexpr int NPAR = 4;  // U, tau0, Cs, r

// Resident blocks per SM of the forward and reverse kernels in float32 (the
// timed precision); float64 leaves the register count to the compiler.
// Measured on the 256x128x32 adjoint (forward / backward ms): the compiler's
// own choice (96 and 168 registers, 5 and 3 blocks) 77.6 / 222.5; 6 and 4
// blocks 72.8 / 211.7; 8 and 4 blocks (64 and 128 registers) 66.7 / 206.2.
#ifndef LBM_ADJ_STEP_MIN_BLOCKS
#define LBM_ADJ_STEP_MIN_BLOCKS 8
#endif
#ifndef LBM_ADJ_REVERSE_MIN_BLOCKS
#define LBM_ADJ_REVERSE_MIN_BLOCKS 4
#endif
template <typename T>
constexpr int adj_step_blocks() {
  return sizeof(T) == 4 ? LBM_ADJ_STEP_MIN_BLOCKS : 1;
}
template <typename T>
constexpr int adj_reverse_blocks() {
  return sizeof(T) == 4 ? LBM_ADJ_REVERSE_MIN_BLOCKS : 1;
}
constexpr double SMAG = 25.456;  // 18 sqrt(2) as the reference writes it (lbm.py:93)

template <typename T> __device__ __forceinline__ T add_rn(T a, T b);
template <> __device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
template <typename T> __device__ __forceinline__ T sub_rn(T a, T b);
template <> __device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// compensated pair (TwoSum), in the precision of the run
template <typename T>
struct Pair {
  T hi, lo;
};
template <typename T>
__device__ __forceinline__ Pair<T> pair_add(Pair<T> a, Pair<T> b) {
  const T s = add_rn(a.hi, b.hi);
  const T bp = sub_rn(s, a.hi);
  const T ap = sub_rn(s, bp);
  const T e = add_rn(sub_rn(a.hi, ap), sub_rn(b.hi, bp));
  const T lo = add_rn(add_rn(a.lo, b.lo), e);
  const T hi = add_rn(s, lo);
  return {hi, sub_rn(lo, sub_rn(hi, s))};
}

// Adds the block's sums of v[0..K) into its slots acc[(block*K + k)*2 + {0, 1}]
// (one block per slot, so launches in stream order accumulate without atomics).
template <typename T, int K>
__device__ __forceinline__ void block_accumulate(const T v[K], T *acc) {
  __shared__ Pair<T> red[BY][K];
  const int lane = threadIdx.x, warp = threadIdx.y;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    Pair<T> x{v[k], T(0)};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      Pair<T> y{__shfl_down_sync(0xffffffffu, x.hi, o), __shfl_down_sync(0xffffffffu, x.lo, o)};
      x = pair_add(x, y);
    }
    if (lane == 0) red[warp][k] = x;
  }
  __syncthreads();
  const int t = warp * BX + lane;
  if (t < K) {
    Pair<T> s = red[0][t];
    for (int w = 1; w < BY; ++w) s = pair_add(s, red[w][t]);
    const size_t slot = ((size_t)block_id() * K + t) * 2;
    const Pair<T> old{acc[slot], acc[slot + 1]};
    const Pair<T> nw = pair_add(old, s);
    acc[slot] = nw.hi;
    acc[slot + 1] = nw.lo;
  }
}

template <typename T>
struct DArgs {
  const T *fin;
  T *fout;
  const T *phi;
  const uint8_t *band;  // per block: 1 when a cell of the block or one of its sources has phi != 0
  const T *Bn, *Gn;  // adjoint of this step's outputs, in the B/G split
  T *Bo, *Go;        // adjoint of its inputs
  T *acc;            // per-block accumulators
  int nx, ny, nz, n;
  T u0, tau0, cs, inv_width;
  T sponge_start, inv_sponge_len, sponge_strength;
  T beta;            // weight of this step's x force in the loss (0: not in it)
  T seed_amp;
};

// periodic neighbour offsets of a cell
struct Nb {
  int xm, xp, ym, yp, zm, zp;  // offsets to x-1, x+1, y-1, ...
};
__device__ __forceinline__ Nb neighbours(int x, int y, int z, int nx, int ny, int nz) {
  Nb o;
  const int nxy = nx * ny;
  o.xm = x == 0 ? nx - 1 : -1;
  o.xp = x == nx - 1 ? 1 - nx : 1;
  o.ym = y == 0 ? (ny - 1) * nx : -nx;
  o.yp = y == ny - 1 ? -(ny - 1) * nx : nx;
  o.zm = z == 0 ? (nz - 1) * nxy : -nxy;
  o.zp = z == nz - 1 ? -(nz - 1) * nxy : nxy;
  return o;
}
// offset from a cell to the cell at (+s) c_q, s = +-1
template <int q, int s>
__device__ __forceinline__ int shift(const Nb &o) {
  const int ex = s * cx(q), ey = s * cy(q), ez = s * cz(q);
  return (ex == 1 ? o.xp : ex == -1 ? o.xm : 0) + (ey == 1 ? o.yp : ey == -1 ? o.ym : 0) +
         (ez == 1 ? o.zp : ez == -1 ? o.zm : 0);
}

template <typename T, int q>
__device__ __forceinline__ T cdot(T ux, T uy, T uz) {
  T s = T(0);
  if (cx(q)) s += T(cx(q)) * ux;
  if (cy(q)) s += T(cy(q)) * uy;
  if (cz(q)) s += T(cz(q)) * uz;
  return s;
}

// feq_q - w_q = w_q (drho + rho (3 s + 4.5 s^2 - 1.5 u^2)), rho = 1 + drho
template <typename T, int q>
__device__ __forceinline__ T dfeq(T drho, T rho, T ux, T uy, T uz, T usq) {
  const T s = cdot<T, q>(ux, uy, uz);
  return T(wq(q)) * (drho + rho * (T(3) * s + T(4.5) * s * s - T(1.5) * usq));
}

// transposed Jacobian of feq(rho, u) applied to e[]: adds to rb and ub.
// By direction pairs (q, opp q = q + 1), with s_opp = -s_q and c_opp = -c_q:
// a pair adds w (e_q + e_opp) to the sums of w e and w e s^2 terms, and
// w (e_q - e_opp) to those of w e c and w e s.
template <typename T>
__device__ __forceinline__ void feq_vjp(const T e[Q], T rho, T ux, T uy, T uz, T &rb, T &ubx, T &uby, T &ubz) {
  const T usq = ux * ux + uy * uy + uz * uz;
  T a0 = T(wq(0)) * e[0], a1x = 0, a1y = 0, a1z = 0, a2x = 0, a2y = 0, a2z = 0, q0 = 0;
  static_for<9>([&](auto kc) {
    constexpr int k = decltype(kc)::value;
    constexpr int q = pq(k);
    const T s = cdot<T, q>(ux, uy, uz);
    const T wp = T(wq(q)) * (e[q] + e[q + 1]);
    const T wm = T(wq(q)) * (e[q] - e[q + 1]);
    a0 += wp;
    q0 += T(3) * s * wm + T(4.5) * s * s * wp;
    const T sp = s * wp;
    if (cx(q)) { a1x += T(cx(q)) * wm; a2x += T(cx(q)) * sp; }
    if (cy(q)) { a1y += T(cy(q)) * wm; a2y += T(cy(q)) * sp; }
    if (cz(q)) { a1z += T(cz(q)) * wm; a2z += T(cz(q)) * sp; }
  });
  rb += a0 + q0 - T(1.5) * usq * a0;
  ubx += rho * (T(3) * a1x + T(9) * a2x - T(3) * ux * a0);
  uby += rho * (T(3) * a1y + T(9) * a2y - T(3) * uy * a0);
  ubz += rho * (T(3) * a1z + T(9) * a2z - T(3) * uz * a0);
}

// The forward arithmetic of one cell, kept for the reverse sweep.
template <typename T>
struct Fwd {
  T fl, sp, sigma, keep;
  T drho, rho, inv, jx, jy, jz, ux, uy, uz, usq;
  T pi[6], pn, c, root, om;
  T drhos, rhos, usx, usy, usz, usqs;
};

// Moments, stress, relaxation time and sponge of one cell from its streamed
// deviations g[] (the production step's pair arithmetic, lbm_device.cuh).
template <typename T>
__device__ __forceinline__ void forward_cell(const DArgs<T> &a, int x, T fl, const T g[Q], Fwd<T> &F) {
  T D[9], M[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    D[k] = g[pq(k)] + g[pq(k) + 1];
    M[k] = g[pq(k)] - g[pq(k) + 1];
  }
  T sum = g[0];
#pragma unroll
  for (int k = 0; k < 9; ++k) sum += D[k];
  F.fl = fl;
  F.drho = sum + T(W_EXCESS);
  F.rho = T(1) + F.drho;
  F.inv = rcp_fast<T>(F.rho);
  F.jx = M[0] + M[3] + M[4] + M[5] + M[6];
  F.jy = M[1] + M[3] - M[4] + M[7] + M[8];
  F.jz = M[2] + M[5] - M[6] + M[7] - M[8];
  F.ux = fl * F.jx * F.inv;
  F.uy = fl * F.jy * F.inv;
  F.uz = fl * F.jz * F.inv;
  const T uxx = F.ux * F.ux, uyy = F.uy * F.uy, uzz = F.uz * F.uz;
  F.usq = uxx + uyy + uzz;
  // Pi_ab = sum c_a c_b (g - feq): deviation pair sums minus the equilibrium's
  // second moments, W2 (drho - 1.5 rho u^2) + 4.5 rho (W2 u_a^2 + W22 (u^2 - u_a^2))
  // on the diagonal and 9 rho W22 u_a u_b off it (lbm_device.cuh, collide())
  const T r45 = T(4.5) * F.rho;
  const T iso = T(W2) * (F.drho - T(1.5) * F.rho * F.usq) + r45 * T(W22) * F.usq;
  const T diag = r45 * T(W2 - W22);
  const T offd = T(9) * F.rho * T(W22);
  F.pi[0] = (D[0] + D[3] + D[4] + D[5] + D[6]) - iso - diag * uxx;
  F.pi[1] = (D[1] + D[3] + D[4] + D[7] + D[8]) - iso - diag * uyy;
  F.pi[2] = (D[2] + D[5] + D[6] + D[7] + D[8]) - iso - diag * uzz;
  F.pi[3] = (D[3] - D[4]) - offd * F.ux * F.uy;
  F.pi[4] = (D[5] - D[6]) - offd * F.ux * F.uz;
  F.pi[5] = (D[7] - D[8]) - offd * F.uy * F.uz;
  F.pn = sqrt_fast<T>(F.pi[0] * F.pi[0] + F.pi[1] * F.pi[1] + F.pi[2] * F.pi[2] +
                     T(2) * (F.pi[3] * F.pi[3] + F.pi[4] * F.pi[4] + F.pi[5] * F.pi[5]));
  F.c = T(SMAG) * a.cs * a.cs;
  F.root = sqrt_fast<T>(a.tau0 * a.tau0 + F.c * F.pn * F.inv);
  F.om = rcp_fast<T>(T(0.5) * (a.tau0 + F.root));
  const T t = fmax(T(0), (T(x) - a.sponge_start) * a.inv_sponge_len);
  F.sp = a.sponge_strength * t * t;
  F.sigma = T(1) - fl * (T(1) - F.sp);
  F.keep = T(1) - F.sigma;
  // rho_s = rho + sigma (1 - rho) = 1 + keep drho
  F.drhos = F.keep * F.drho;
  F.rhos = T(1) + F.drhos;
  F.usx = F.ux + F.sigma * (a.u0 * fl - F.ux);
  F.usy = F.keep * F.uy;
  F.usz = F.keep * F.uz;
  F.usqs = F.usx * F.usx + F.usy * F.usy + F.usz * F.usz;
}

// Streamed deviations g[] of cell idx. BAND: the bounce-back blend with phi at
// the sources; otherwise the plain pull.
template <typename T, bool BAND>
__device__ __forceinline__ void stream_cell(const DArgs<T> &a, int idx, const Nb &o, T g[Q]) {
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    const int s = idx + shift<q, -1>(o);
    const T p = __ldg(a.fin + q * a.n + s);
    if (BAND && q != 0) {
      const T ph = __ldg(a.phi + s);
      const T b = __ldg(a.fin + opp(q) * a.n + idx);
      g[q] = p + ph * (b - p);
    } else {
      g[q] = p;
    }
  });
}

// x force of one band cell from its bounced values: sum_q -c_qx phi_q fl 2 (w + b)
template <typename T>
__device__ __forceinline__ T cell_force(const DArgs<T> &a, int idx, const Nb &o, T fl) {
  T force = T(0);
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    if (q != 0 && cx(q) != 0) {
      const T ph = __ldg(a.phi + idx + shift<q, -1>(o));
      const T b = __ldg(a.fin + opp(q) * a.n + idx);
      force += T(-cx(q)) * ph * fl * T(2) * (T(wq(q)) + b);
    }
  });
  return force;
}

template <typename T, bool BAND>
__device__ __forceinline__ T step_cell(const DArgs<T> &a, int x, int idx, const Nb &o) {
  T g[Q];
  stream_cell<T, BAND>(a, idx, o, g);
  const T fl = BAND ? T(1) - __ldg(a.phi + idx) : T(1);
  Fwd<T> F;
  forward_cell(a, x, fl, g, F);
  // out = feq(rho_s, u_s) + keep (post - feq) = feq_s + keep (1 - om) (g - feq),
  // the equilibria in the pair form w (A +- B) (lbm_device.cuh, eq_pair);
  // with sigma = 0 (fluid outside the sponge) feq_s is feq itself
  const T alpha = F.keep * (T(1) - F.om);
  const EqBase<T> e = eq_base<T>(F.drho, F.rho, F.ux, F.uy, F.uz);
  const EqBase<T> es = F.sigma == T(0) ? e : eq_base<T>(F.drhos, F.rhos, F.usx, F.usy, F.usz);
  const T usx = F.sigma == T(0) ? F.ux : F.usx, usy = F.sigma == T(0) ? F.uy : F.usy,
          usz = F.sigma == T(0) ? F.uz : F.usz;
  {
    const T f0 = T(wq(0)) * e.base;
    a.fout[idx] = T(wq(0)) * es.base + alpha * (g[0] - f0);
  }
  static_for<9>([&](auto kc) {
    constexpr int k = decltype(kc)::value;
    constexpr int q = pq(k);
    const T w = T(wq(q));
    T A, B, As, Bs;
    eq_pair<T, k>(e, F.ux, F.uy, F.uz, A, B);
    eq_pair<T, k>(es, usx, usy, usz, As, Bs);
    a.fout[q * a.n + idx] = w * (As + Bs) + alpha * (g[q] - w * (A + B));
    a.fout[(q + 1) * a.n + idx] = w * (As - Bs) + alpha * (g[q + 1] - w * (A - B));
  });
  return BAND && a.beta != T(0) ? cell_force(a, idx, o, fl) : T(0);
}

// Forward step f_{t-1} -> f_t; when beta != 0 also the step's x force.
template <typename T>
__global__ void __launch_bounds__(BX * BY, adj_step_blocks<T>()) diff_step_kernel(const __grid_constant__ DArgs<T> a) {
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
  const bool band = a.band[block_id()] != 0;
  T force = 0;
  if (x < a.nx && y < a.ny) {
    const int idx = (z * a.ny + y) * a.nx + x;
    const Nb o = neighbours(x, y, z, a.nx, a.ny, a.nz);
    force = band ? step_cell<T, true>(a, x, idx, o) : step_cell<T, false>(a, x, idx, o);
  }
  if (a.beta != T(0)) {
    T v[1] = {force};
    block_accumulate<T, 1>(v, a.acc);
  }
}

// Reverse of step t for one cell: lambda_t (B/G split) -> lambda_{t-1} (B/G
// split) and the cell's parameter gradients.
template <typename T, bool BAND>
__device__ __forceinline__ void adjoint_cell(const DArgs<T> &a, int x, int idx, const Nb &o, T grad[NPAR]) {
  T g[Q];
  stream_cell<T, BAND>(a, idx, o, g);
  const T phx = BAND ? __ldg(a.phi + idx) : T(0);
  Fwd<T> F;
  forward_cell(a, x, T(1) - phx, g, F);
  // g <- ne = g - feq(rho, u), feq in the pair form of step_cell
  {
    const EqBase<T> e = eq_base<T>(F.drho, F.rho, F.ux, F.uy, F.uz);
    g[0] -= T(wq(0)) * e.base;
    static_for<9>([&](auto kc) {
      constexpr int k = decltype(kc)::value;
      constexpr int q = pq(k);
      T A, B;
      eq_pair<T, k>(e, F.ux, F.uy, F.uz, A, B);
      g[q] -= T(wq(q)) * (A + B);
      g[q + 1] -= T(wq(q)) * (A - B);
    });
  }
  // adjoint of the outputs f_t[q](x)
  T ob[Q];
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    const T gin = a.Gn[q * a.n + idx + shift<q, 1>(o)];
    ob[q] = (BAND && q != 0) ? a.Bn[q * a.n + idx] + gin : gin;
  });
  // out = feq(rho_s, u_s) + keep (1 - om) ne
  T rsb = 0, usbx = 0, usby = 0, usbz = 0;
  feq_vjp<T>(ob, F.rhos, F.usx, F.usy, F.usz, rsb, usbx, usby, usbz);
  T s1 = 0;  // sum ob ne
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    s1 += ob[q] * g[q];
  });
  const T one_om = T(1) - F.om;
  const T alpha = F.keep * one_om;
  const T kb = one_om * s1;     // d/d keep
  const T omb = -F.keep * s1;   // d/d om
  // sponge blend: rho_s, u_s, keep = 1 - sigma
  T sigb = -kb - rsb * F.drho + usbx * (a.u0 * F.fl - F.ux) - usby * F.uy - usbz * F.uz;
  T rhob = rsb * F.keep;
  T uxb = usbx * F.keep, uyb = usby * F.keep, uzb = usbz * F.keep;
  grad[0] += usbx * F.sigma * F.fl;
  T flb = usbx * F.sigma * a.u0 - sigb * (T(1) - F.sp);
  // om = 1/tau, tau = (tau0 + root)/2, root^2 = tau0^2 + c pn / rho
  const T taub = -omb * F.om * F.om;
  const T innerb = taub * rcp_fast<T>(T(4) * F.root);
  grad[1] += T(0.5) * taub + innerb * T(2) * a.tau0;
  grad[2] += innerb * F.pn * F.inv * T(SMAG) * T(2) * a.cs;
  const T pnb = innerb * F.c * F.inv;
  rhob -= innerb * F.c * F.pn * F.inv * F.inv;
  T pib[6] = {0, 0, 0, 0, 0, 0};
  if (F.pn > T(0)) {
    const T s = pnb * rcp_fast<T>(F.pn);
    pib[0] = s * F.pi[0];
    pib[1] = s * F.pi[1];
    pib[2] = s * F.pi[2];
    pib[3] = T(2) * s * F.pi[3];
    pib[4] = T(2) * s * F.pi[4];
    pib[5] = T(2) * s * F.pi[5];
  }
  // ne = g - feq: gb = alpha ob + sum_ab c_a c_b pib_ab, and feq's adjoint is
  // -gb; c_a c_b is the same for q and opp q, so each pair forms it once
  ob[0] = alpha * ob[0];
  static_for<9>([&](auto kc) {
    constexpr int k = decltype(kc)::value;
    constexpr int q = pq(k);
    T m = 0;
    if (cx(q)) m += pib[0];
    if (cy(q)) m += pib[1];
    if (cz(q)) m += pib[2];
    if (cx(q) && cy(q)) m += T(cx(q) * cy(q)) * pib[3];
    if (cx(q) && cz(q)) m += T(cx(q) * cz(q)) * pib[4];
    if (cy(q) && cz(q)) m += T(cy(q) * cz(q)) * pib[5];
    ob[q] = alpha * ob[q] + m;
    ob[q + 1] = alpha * ob[q + 1] + m;
  });
  {
    T r = 0, bx = 0, by = 0, bz = 0;
    feq_vjp<T>(ob, F.rho, F.ux, F.uy, F.uz, r, bx, by, bz);
    rhob -= r;
    uxb -= bx;
    uyb -= by;
    uzb -= bz;
  }
  // u = fl j / rho
  const T jxb = uxb * F.fl * F.inv, jyb = uyb * F.fl * F.inv, jzb = uzb * F.fl * F.inv;
  rhob -= (uxb * F.ux + uyb * F.uy + uzb * F.uz) * F.inv;
  flb += (uxb * F.jx + uyb * F.jy + uzb * F.jz) * F.inv;
  // moments, streaming and bounce-back (and the drag); outputs. The
  // momentum part c_q . jb is formed once per pair (c_opp = -c_q).
  T cj[9];
  static_for<9>([&](auto kc) {
    constexpr int k = decltype(kc)::value;
    cj[k] = cdot<T, pq(k)>(jxb, jyb, jzb);
  });
  T rb = 0;
  static_for<Q>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    const T gq = q == 0 ? ob[0] + rhob : (q & 1) ? (ob[q] + rhob) + cj[(q - 1) / 2] : (ob[q] + rhob) - cj[(q - 1) / 2];
    if (!BAND || q == 0) {
      a.Go[q * a.n + idx] = gq;
    } else {
      const int s = idx + shift<q, -1>(o);
      const T ph = __ldg(a.phi + s);
      const T b = __ldg(a.fin + opp(q) * a.n + idx);
      const T p = __ldg(a.fin + q * a.n + s);
      T bb = gq * ph;
      T phb = gq * (b - p);
      if (cx(q) != 0 && a.beta != T(0)) {
        const T d = a.beta * T(-cx(q)) * T(2);
        const T bf = T(wq(q)) + b;  // the bounced population itself
        bb += d * ph * F.fl;
        phb += d * F.fl * bf;
        flb += d * ph * bf;
      }
      a.Go[q * a.n + idx] = gq * (T(1) - ph);
      a.Bo[opp(q) * a.n + idx] = bb;
      rb += phb * T(2) * ph * (T(1) - ph) * a.inv_width;
    }
  });
  if (BAND) grad[3] += rb - flb * T(2) * phx * (T(1) - phx) * a.inv_width;
}

template <typename T>
__global__ void __launch_bounds__(BX * BY, adj_reverse_blocks<T>())
diff_adjoint_kernel(const __grid_constant__ DArgs<T> a) {
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
  const bool band = a.band[block_id()] != 0;
  T grad[NPAR] = {0, 0, 0, 0};
  if (x < a.nx && y < a.ny) {
    const int idx = (z * a.ny + y) * a.nx + x;
    const Nb o = neighbours(x, y, z, a.nx, a.ny, a.nz);
    if (band) adjoint_cell<T, true>(a, x, idx, o, grad);
    else adjoint_cell<T, false>(a, x, idx, o, grad);
  }
  block_accumulate<T, NPAR>(grad, a.acc);
}

// Start state f_0 = feq(1, (U fl, A U fl sin(2 pi x/nx) cos(2 pi z/nz), 0)) (lbm.py:383-394).
template <typename T>
__device__ __forceinline__ void init_velocity(const DArgs<T> &a, int x, int z, T fl, T &ux, T &uy, T &wave) {
  wave = a.seed_amp * T(sin(6.283185307179586 * (double)x / (double)a.nx) *
                        cos(6.283185307179586 * (double)z / (double)a.nz));
  ux = a.u0 * fl;
  uy = wave * a.u0 * fl;
}

template <typename T>
__global__ void diff_init_kernel(const __grid_constant__ DArgs<T> a) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < a.n; idx += gridDim.x * blockDim.x) {
    const int x = idx % a.nx, z = idx / (a.nx * a.ny);
    T ux, uy, wave;
    init_velocity(a, x, z, T(1) - a.phi[idx], ux, uy, wave);
    const T usq = ux * ux + uy * uy;
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      a.fout[q * a.n + idx] = dfeq<T, q>(T(0), T(1), ux, uy, T(0), usq);
    });
  }
}

// gradient contributions of the start state, from lambda_0 (B/G split)
template <typename T>
__global__ void __launch_bounds__(BX * BY) diff_init_adjoint_kernel(const __grid_constant__ DArgs<T> a) {
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
  const bool band = a.band[block_id()] != 0;
  T grad[NPAR] = {0, 0, 0, 0};
  if (x < a.nx && y < a.ny) {
    const int idx = (z * a.ny + y) * a.nx + x;
    const Nb o = neighbours(x, y, z, a.nx, a.ny, a.nz);
    T e[Q];
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      const T gin = a.Gn[q * a.n + idx + shift<q, 1>(o)];
      e[q] = (band && q != 0) ? a.Bn[q * a.n + idx] + gin : gin;
    });
    const T phx = a.phi[idx], fl = T(1) - phx;
    T ux, uy, wave;
    init_velocity(a, x, z, fl, ux, uy, wave);
    T rb = 0, uxb = 0, uyb = 0, uzb = 0;
    feq_vjp<T>(e, T(1), ux, uy, T(0), rb, uxb, uyb, uzb);
    grad[0] = uxb * fl + uyb * wave * fl;
    const T flb = uxb * a.u0 + uyb * wave * a.u0;
    grad[3] = -flb * T(2) * phx * (T(1) - phx) * a.inv_width;
  }
  block_accumulate<T, NPAR>(grad, a.acc);
}

template <typename T>
__global__ void phi_kernel(T *phi, int nx, int ny, int n, T ox, T oy, T r, T inv_width) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const int x = idx % nx, y = (idx / nx) % ny;
    const T dx = T(x) - ox, dy = T(y) - oy;
    phi[idx] = T(0.5) * (T(1) + tanh((r - sqrt(dx * dx + dy * dy)) * inv_width));
  }
}

// Band flags: a cell with phi != 0 marks its own block and the blocks of the
// 18 cells that pull from it (x + c_q, periodic). Every flag written is 1, so
// the concurrent stores need no atomics.
template <typename T>
__global__ void band_kernel(const T *phi, uint8_t *band, int nx, int ny, int nz, int gx, int gy) {
  const int n = nx * ny * nz;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    if (phi[idx] == T(0)) continue;
    const int x = idx % nx, y = (idx / nx) % ny, z = idx / (nx * ny);
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      int xs = x + cx(q), ys = y + cy(q), zs = z + cz(q);
      xs += xs < 0 ? nx : 0;
      xs -= xs >= nx ? nx : 0;
      ys += ys < 0 ? ny : 0;
      ys -= ys >= ny ? ny : 0;
      zs += zs < 0 ? nz : 0;
      zs -= zs >= nz ? nz : 0;
      band[((size_t)zs * gy + ys / BY) * gx + xs / BX] = 1;
    });
  }
}

}  // namespace lbma

// ---------------------------------------------------------------------------
// Host driver

struct lbm_adj {
  lbm_adj_config cfg;
  double par[4];     // U, tau0, Cs, r
  int64_t n;
  size_t esz;        // bytes per value (4 or 8)
  size_t state;      // bytes per population state (19 n values)
  void *phi = nullptr;
  uint8_t *band = nullptr;  // per-block obstacle-band flags
  std::vector<void *> ck;   // checkpoints f_{mK}, m = 0..M
  std::vector<void *> seg;  // recomputed states of one segment
  void *tmp[2] = {nullptr, nullptr};
  void *adj[4] = {nullptr, nullptr, nullptr, nullptr};  // B, G (in), B, G (out)
  void *acc = nullptr;      // per-block accumulators (NPAR pairs per block)
  int64_t nblocks = 0;
  dim3 grid, block;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  double loss = 0.0;
  double force_sum = 0.0;
  double fwd_ms = 0.0, bwd_ms = 0.0;
  int forward_done = 0;
  int64_t bytes = 0;
};

namespace {

lbm_status afail(lbm_status s, const std::string &msg) {
  lbmh::set_last_error(msg);
  return s;
}

#define ACUDA(call)                                                                      \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) return afail(LBM_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

int num_segments(const lbm_adj_config &c) { return (c.steps + c.checkpoint - 1) / c.checkpoint; }

template <typename T>
lbma::DArgs<T> dargs(const lbm_adj *h) {
  lbma::DArgs<T> a{};
  const lbm_adj_config &c = h->cfg;
  a.phi = static_cast<const T *>(h->phi);
  a.band = h->band;
  a.nx = c.nx;
  a.ny = c.ny;
  a.nz = c.nz;
  a.n = (int)h->n;
  a.u0 = (T)h->par[0];
  a.tau0 = (T)h->par[1];
  a.cs = (T)h->par[2];
  a.inv_width = (T)(1.0 / c.width);
  a.sponge_start = (T)c.sponge_start;
  a.inv_sponge_len = (T)(1.0 / ((double)c.nx - c.sponge_start));
  a.sponge_strength = (T)c.sponge_strength;
  a.seed_amp = (T)c.seed_amp;
  a.acc = static_cast<T *>(h->acc);
  return a;
}

double beta_of(const lbm_adj *h) {
  const lbm_adj_config &c = h->cfg;
  const double nl = (double)(c.steps - c.loss_start + 1);
  const double u = h->par[0];
  return 1.0 / (nl * 0.5 * u * u * c.diameter * c.nz);
}

// sum of the per-block pairs of accumulator k (K per block), in double on the host
template <typename T>
lbm_status read_acc(const lbm_adj *h, int K, double *out) {
  std::vector<T> v((size_t)h->nblocks * K * 2);
  ACUDA(cudaMemcpy(v.data(), h->acc, v.size() * sizeof(T), cudaMemcpyDeviceToHost));
  for (int k = 0; k < K; ++k) {
    long double s = 0.0L;
    for (int64_t b = 0; b < h->nblocks; ++b)
      s += (long double)v[((size_t)b * K + k) * 2] + (long double)v[((size_t)b * K + k) * 2 + 1];
    out[k] = (double)s;
  }
  return LBM_OK;
}

template <typename T>
lbm_status phi_and_init(lbm_adj *h, void *f0) {
  const lbm_adj_config &c = h->cfg;
  const int g = lbmk::cell_grid(h->n);
  lbma::phi_kernel<T><<<g, 256>>>(static_cast<T *>(h->phi), c.nx, c.ny, (int)h->n, (T)c.ox, (T)c.oy,
                                  (T)h->par[3], (T)(1.0 / c.width));
  ACUDA(cudaMemsetAsync(h->band, 0, (size_t)h->nblocks));
  lbma::band_kernel<T><<<g, 256>>>(static_cast<const T *>(h->phi), h->band, c.nx, c.ny, c.nz, (int)h->grid.x,
                                   (int)h->grid.y);
  lbma::DArgs<T> a = dargs<T>(h);
  a.fout = static_cast<T *>(f0);
  lbma::diff_init_kernel<T><<<g, 256>>>(a);
  ACUDA(cudaGetLastError());
  return LBM_OK;
}

template <typename T>
void launch_fwd(lbm_adj *h, const void *fin, void *fout, double beta) {
  lbma::DArgs<T> a = dargs<T>(h);
  a.fin = static_cast<const T *>(fin);
  a.fout = static_cast<T *>(fout);
  a.beta = (T)beta;
  lbma::diff_step_kernel<T><<<h->grid, h->block>>>(a);
}

template <typename T>
lbm_status forward(lbm_adj *h) {
  const lbm_adj_config &c = h->cfg;
  ACUDA(cudaEventRecord(h->ev[0]));
  lbm_status st = phi_and_init<T>(h, h->ck[0]);
  if (st != LBM_OK) return st;
  ACUDA(cudaMemset(h->acc, 0, (size_t)h->nblocks * lbma::NPAR * 2 * h->esz));
  const void *cur = h->ck[0];
  for (int t = 1; t <= c.steps; ++t) {
    void *dst = t % c.checkpoint == 0 ? h->ck[t / c.checkpoint] : h->tmp[t & 1];
    launch_fwd<T>(h, cur, dst, t >= c.loss_start ? 1.0 : 0.0);
    cur = dst;
  }
  ACUDA(cudaGetLastError());
  ACUDA(cudaEventRecord(h->ev[1]));
  ACUDA(cudaEventSynchronize(h->ev[1]));
  float ms = 0.f;
  ACUDA(cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]));
  h->fwd_ms = ms;
  // the forward kernel keeps one accumulator (the x force) per block
  double s[1];
  st = read_acc<T>(h, 1, s);
  if (st != LBM_OK) return st;
  h->force_sum = s[0];
  h->loss = s[0] * beta_of(h);
  h->forward_done = 1;
  return LBM_OK;
}

template <typename T>
lbm_status backward(lbm_adj *h, double grad[4]) {
  const lbm_adj_config &c = h->cfg;
  const double beta = beta_of(h);
  ACUDA(cudaEventRecord(h->ev[2]));
  ACUDA(cudaMemset(h->acc, 0, (size_t)h->nblocks * lbma::NPAR * 2 * h->esz));
  ACUDA(cudaMemset(h->adj[0], 0, h->state));
  ACUDA(cudaMemset(h->adj[1], 0, h->state));
  void *Bn = h->adj[0], *Gn = h->adj[1], *Bo = h->adj[2], *Go = h->adj[3];
  const int M = num_segments(c);
  for (int m = M - 1; m >= 0; --m) {
    const int t0 = m * c.checkpoint;                        // checkpointed state f_{t0}
    const int t1 = std::min((m + 1) * c.checkpoint, c.steps);  // last step of the segment
    // recompute f_{t0+1} .. f_{t1-1}
    h->seg[0] = h->ck[m];
    for (int t = t0 + 1; t < t1; ++t) launch_fwd<T>(h, h->seg[t - 1 - t0], h->seg[t - t0], 0.0);
    for (int t = t1; t > t0; --t) {
      lbma::DArgs<T> a = dargs<T>(h);
      a.fin = static_cast<const T *>(h->seg[t - 1 - t0]);
      a.Bn = static_cast<const T *>(Bn);
      a.Gn = static_cast<const T *>(Gn);
      a.Bo = static_cast<T *>(Bo);
      a.Go = static_cast<T *>(Go);
      a.beta = t >= c.loss_start ? (T)beta : (T)0;
      lbma::diff_adjoint_kernel<T><<<h->grid, h->block>>>(a);
      std::swap(Bn, Bo);
      std::swap(Gn, Go);
    }
  }
  {
    lbma::DArgs<T> a = dargs<T>(h);
    a.Bn = static_cast<const T *>(Bn);
    a.Gn = static_cast<const T *>(Gn);
    lbma::diff_init_adjoint_kernel<T><<<h->grid, h->block>>>(a);
  }
  ACUDA(cudaGetLastError());
  ACUDA(cudaEventRecord(h->ev[3]));
  ACUDA(cudaEventSynchronize(h->ev[3]));
  float ms = 0.f;
  ACUDA(cudaEventElapsedTime(&ms, h->ev[2], h->ev[3]));
  h->bwd_ms = ms;
  lbm_status st = read_acc<T>(h, lbma::NPAR, grad);
  if (st != LBM_OK) return st;
  // the loss's normalisation 1/(0.5 U^2 D nz) also depends on U
  grad[0] += -2.0 * h->loss / h->par[0];
  return LBM_OK;
}

void release(lbm_adj *h) {
  cudaFree(h->phi);
  cudaFree(h->band);
  for (void *p : h->ck) cudaFree(p);
  for (size_t i = 1; i < h->seg.size(); ++i) cudaFree(h->seg[i]);
  for (void *&p : h->tmp) cudaFree(p);
  for (void *&p : h->adj) cudaFree(p);
  cudaFree(h->acc);
  for (cudaEvent_t &e : h->ev)
    if (e) cudaEventDestroy(e);
}

}  // namespace

extern "C" {

lbm_status lbm_adj_create(const lbm_adj_config *cfg, lbm_adj **out) {
  if (!cfg || !out) return afail(LBM_ERR_ARG, "null argument");
  *out = nullptr;
  const lbm_adj_config &c = *cfg;
  if (c.nx < 2 || c.ny < 2 || c.nz < 1 || (int64_t)c.nx * c.ny * c.nz > (int64_t)INT32_MAX / 19)
    return afail(LBM_ERR_ARG, "lattice sizes out of range");
  if (c.precision != LBM_F32 && c.precision != LBM_F64) return afail(LBM_ERR_ARG, "precision must be LBM_F32 or LBM_F64");
  if (c.steps < 1 || c.checkpoint < 1 || c.loss_start < 1 || c.loss_start > c.steps)
    return afail(LBM_ERR_ARG, "need steps >= 1, checkpoint >= 1 and 1 <= loss_start <= steps");
  if (!(c.width > 0.0) || !(c.diameter > 0.0) || !(c.sponge_start < c.nx))
    return afail(LBM_ERR_ARG, "need width > 0, diameter > 0 and sponge_start < nx");
  ACUDA(cudaSetDevice(c.device));
  lbm_adj *h = new (std::nothrow) lbm_adj();
  if (!h) return afail(LBM_ERR_ARG, "out of host memory");
  h->cfg = c;
  h->par[0] = c.u0;
  h->par[1] = c.tau0;
  h->par[2] = c.cs;
  h->par[3] = c.r;
  h->n = (int64_t)c.nx * c.ny * c.nz;
  h->esz = c.precision == LBM_F64 ? 8 : 4;
  h->state = (size_t)19 * h->n * h->esz;
  h->block = dim3(lbmk::BX, lbmk::BY);
  h->grid = dim3((c.nx + lbmk::BX - 1) / lbmk::BX, (c.ny + lbmk::BY - 1) / lbmk::BY, c.nz);
  h->nblocks = (int64_t)h->grid.x * h->grid.y * h->grid.z;
  const int M = num_segments(c);
  auto alloc = [&](void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) h->bytes += (int64_t)bytes;
    return e;
  };
  cudaError_t e = alloc(&h->phi, (size_t)h->n * h->esz);
  if (e == cudaSuccess) e = alloc((void **)&h->band, (size_t)h->nblocks);
  h->ck.assign(M + 1, nullptr);
  for (int m = 0; m <= M && e == cudaSuccess; ++m) e = alloc(&h->ck[m], h->state);
  h->seg.assign(c.checkpoint, nullptr);
  for (int i = 1; i < c.checkpoint && e == cudaSuccess; ++i) e = alloc(&h->seg[i], h->state);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = alloc(&h->tmp[i], h->state);
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = alloc(&h->adj[i], h->state);
  if (e == cudaSuccess) e = alloc(&h->acc, (size_t)h->nblocks * lbma::NPAR * 2 * h->esz);
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreate(&h->ev[i]);
  if (e != cudaSuccess) {
    release(h);
    delete h;
    return afail(LBM_ERR_CUDA, std::string("lbm_adj_create: ") + cudaGetErrorString(e));
  }
  *out = h;
  return LBM_OK;
}

lbm_status lbm_adj_destroy(lbm_adj *h) {
  if (!h) return LBM_OK;
  cudaSetDevice(h->cfg.device);
  release(h);
  delete h;
  return LBM_OK;
}

lbm_status lbm_adj_set_params(lbm_adj *h, const double par[4]) {
  if (!h || !par) return afail(LBM_ERR_ARG, "null argument");
  if (!(par[0] != 0.0) || !(par[1] > 0.5) || !(par[2] >= 0.0) || !(par[3] >= 0.0))
    return afail(LBM_ERR_ARG, "need U != 0, tau0 > 1/2, Cs >= 0, r >= 0");
  for (int k = 0; k < 4; ++k) h->par[k] = par[k];
  h->forward_done = 0;
  return LBM_OK;
}

lbm_status lbm_adj_forward(lbm_adj *h, double *loss) {
  lbmh::Range range_("lbm_adj_forward");
  if (!h || !loss) return afail(LBM_ERR_ARG, "null argument");
  ACUDA(cudaSetDevice(h->cfg.device));
  lbm_status st = h->cfg.precision == LBM_F64 ? forward<double>(h) : forward<float>(h);
  if (st != LBM_OK) return st;
  *loss = h->loss;
  return std::isfinite(h->loss) ? LBM_OK : afail(LBM_ERR_NONFINITE, "loss is not finite");
}

lbm_status lbm_adj_backward(lbm_adj *h, double grad[4]) {
  lbmh::Range range_("lbm_adj_backward");
  if (!h || !grad) return afail(LBM_ERR_ARG, "null argument");
  if (!h->forward_done) return afail(LBM_ERR_STATE, "lbm_adj_backward needs lbm_adj_forward with the current parameters");
  ACUDA(cudaSetDevice(h->cfg.device));
  return h->cfg.precision == LBM_F64 ? backward<double>(h, grad) : backward<float>(h, grad);
}

lbm_status lbm_adj_state(lbm_adj *h, int32_t step, void *host) {
  if (!h || !host) return afail(LBM_ERR_ARG, "null argument");
  if (!h->forward_done) return afail(LBM_ERR_STATE, "no forward run");
  if (step < 0 || step > h->cfg.steps || step % h->cfg.checkpoint != 0)
    return afail(LBM_ERR_ARG, "step must be a checkpointed step (a multiple of the checkpoint interval)");
  ACUDA(cudaSetDevice(h->cfg.device));
  ACUDA(cudaMemcpy(host, h->ck[step / h->cfg.checkpoint], h->state, cudaMemcpyDeviceToHost));
  // the run keeps deviations f_q - w_q: add the weights back
  const int64_t n = h->n;
  for (int q = 0; q < lbmk::Q; ++q) {
    if (h->cfg.precision == LBM_F64) {
      double *f = static_cast<double *>(host) + (size_t)q * n;
      for (int64_t i = 0; i < n; ++i) f[i] += (double)lbmk::wq(q);
    } else {
      float *f = static_cast<float *>(host) + (size_t)q * n;
      for (int64_t i = 0; i < n; ++i) f[i] += lbmk::wq(q);
    }
  }
  return LBM_OK;
}

lbm_status lbm_adj_info(lbm_adj *h, double out[4]) {
  if (!h || !out) return afail(LBM_ERR_ARG, "null argument");
  out[0] = h->fwd_ms;
  out[1] = h->bwd_ms;
  out[2] = h->force_sum;
  out[3] = (double)h->bytes;
  return LBM_OK;
}

}  // extern "C"
