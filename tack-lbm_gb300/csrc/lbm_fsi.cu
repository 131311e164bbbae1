// lbm_fsi.cu - the cantilever-wing FSI step (tack-lbm fsi.py:25-186) and its C ABI.
//
// An elastic NACA 0012 wing from the root plane (a mirror below z = 0) to
// z = span: every lattice layer z has its own plunge h, pitch alpha and their
// rates, given by the caller's structural model each step. Per step:
//   * fsi_mask_kernel evaluates each cell's layer section test into a byte
//     mask (fsi.py:35-47): float64 results, with a float32 prefilter that
//     decides the points away from the outline (lbm_naca.cuh);
//   * fsi_step_kernel (float32 populations on A/B buffers f[q*n + idx]):
//     inflow at x = 0 from the free-stream equilibrium, zero-gradient outflow
//     at x = nx - 1, periodic y, mirror planes below z = 0 and above
//     z = nz - 1; moving-wall bounce-back, second order on wetted links by the
//     interpolated (Bouzidi) rule with the wall's place on the link found by
//     six bisection steps of the float64 section test (fsi.py:49-60,
//     110-126); the momentum exchange relative to the fluid at rest (fsi.py:
//     128-135), reduced per block (all of a block's cells share a layer) and
//     added to the layer's float64 totals; the collision; the sponge, which
//     settles density and the non-equilibrium part while solid cells take the
//     wall velocity (fsi.py:158-172); report fields ux, uy, uz, p, vmag.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "lbm_device.cuh"
#include "lbm_host.h"
#include "lbm_naca.cuh"

namespace lbmf {

using namespace lbmk;

// per layer: h, alpha, dh/dt, dalpha/dt, cos alpha, sin alpha
constexpr int KIN = 6;

struct FsiArgs {
  const float *fin;
  float *fout;
  const uint8_t *mask;
  const double *kin;
  const NacaF *naca;   // per layer: the float32 prefilter (reach < 0 past the span)
  const float4 *kinf;  // per layer: h, dh/dt, dalpha/dt as float32
  double *load;  // 3 per layer
  float *fld[5];
  int nx, ny, nz, n;
  double chord, x_ea, y_ea, ea, span;
  float x_eaf, y_eaf;  // the elastic axis in float32 for the per-cell arithmetic
  float u0, sponge_start, inv_sponge_len, sponge_strength;
  float omega_bgk, tau0, smag_c, magic;
};

// Slot q of cell e in an A/B buffer: FLAT (lattices with 19 n < 2^32) forms
// a 32-bit element offset from the base, else a 64-bit one. The flat form
// takes the step kernel from 92 to 80 registers (6 blocks per SM instead of
// 5) and the coupled step on the 256x128x104 wing from 0.246-0.250 to
// 0.236-0.242 ms of GPU timeline.
template <bool FLAT, typename P>
__device__ __forceinline__ P *fsi_at(P *f, const FsiArgs &a, int q, int e) {
  if (FLAT) return f + (uint32_t)((uint32_t)q * (uint32_t)a.n + (uint32_t)e);
  return f + (size_t)q * a.n + e;
}

__device__ __forceinline__ bool section64(const FsiArgs &a, double x, double y, int z) {
  const double *k = a.kin + KIN * z;
  const double dx = x - a.x_ea, dy = y - (a.y_ea + k[0]);
  const double s = dx * k[4] - dy * k[5], t = dx * k[5] + dy * k[4];
  const double xc = s / a.chord + a.ea;
  const double c = fmin(fmax(xc, 0.0), 1.0);
  const double half = 0.6 * a.chord * (0.2969 * sqrt(c) - 0.1260 * c - 0.3516 * c * c + 0.2843 * c * c * c -
                                       0.1036 * c * c * c * c);
  return xc >= 0.0 && xc <= 1.0 && fabs(t) < half && (double)z + 0.5 < a.span;
}

// the section test at (x, y), both exactly representable in float32 (lattice
// points, and the k/64 points of the wall bisection)
__device__ __forceinline__ bool section(const FsiArgs &a, float x, float y, int z) {
  const int r = naca_prefilter(a.naca[z], x, y);
  return r != 0 ? r > 0 : section64(a, (double)x, (double)y, z);
}

__global__ void fsi_mask_kernel(const __grid_constant__ FsiArgs a, uint8_t *mask) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < a.n; idx += gridDim.x * blockDim.x) {
    const int x = idx % a.nx, y = (idx / a.nx) % a.ny, z = idx / (a.nx * a.ny);
    mask[idx] = section(a, (float)x, (float)y, z) ? 1 : 0;
  }
}

// the wall's place on the link from (x, y, z) toward (x - cx, y - cy, zs), as a fraction
// (the bisection's points k/64 and the points x - mid c_q are exact in
// float32, so float32 carries it with the float64 results of the test)
__device__ __forceinline__ float wall_fraction(const FsiArgs &a, int x, int y, int z, int cxq, int cyq, int zs) {
  float lo = 0.f, hi = 1.f;
  for (int it = 0; it < 6; ++it) {
    const float mid = 0.5f * (lo + hi);
    const bool in = section(a, (float)x - mid * (float)cxq, (float)y - mid * (float)cyq, mid >= 0.5f ? zs : z);
    if (in) hi = mid;
    else lo = mid;
  }
  return 0.5f * (lo + hi);
}

// The interpolated bounce-back of one wetted link, a fluid cell (x, y, z)
// whose source (x - c_q, zs) lies in the wing (fsi.py:110-135): the wall's
// place on the link by bisection, the bounced value (far-wall form for
// delta >= 1/2, near-wall form with the cell behind otherwise) and the
// link's momentum exchange added to (fx, fy, mz). Out of line on purpose:
// few links are wetted, and inlining the bisection with its float64
// fallback into all 18 directions bloats the kernel's common path.
__device__ __noinline__ float wetted_link(const FsiArgs &a, int x, int y, int z, int zs, int idx, int q, int o,
                                          int cxq, int cyq, int czq, float w, float bounced, float &fx, float &fy,
                                          float &mz) {
  const float4 k = a.kinf[zs];
  const float kh = k.x, kdh = k.y, kda = k.z;
  const float df = wall_fraction(a, x, y, z, cxq, cyq, zs);
  const float px = (float)x - df * (float)cxq, py = (float)y - df * (float)cyq;
  const float cu = (float)cxq * (kda * (py - a.y_eaf - kh)) + (float)cyq * (kdh - kda * (px - a.x_eaf));
  float back = bounced + 6.f * w * ((float)cxq * (kda * ((float)y - 0.5f * (float)cyq - a.y_eaf - kh)) +
                                    (float)cyq * (kdh - kda * ((float)x - 0.5f * (float)cxq - a.x_eaf)));
  if (df >= 0.5f) {
    back = (bounced + (2.f * df - 1.f) * *fsi_at<false>(a.fin, a, q, idx) + 6.f * w * cu) / (2.f * df);
  } else {
    int xn = x + cxq;
    xn += xn < 0 ? a.nx : 0;
    xn -= xn >= a.nx ? a.nx : 0;
    int yn = y + cyq;
    yn += yn < 0 ? a.ny : 0;
    yn -= yn >= a.ny ? a.ny : 0;
    const int zn = z + czq;
    const int zc = zn < 0 ? 0 : (zn > a.nz - 1 ? a.nz - 1 : zn);
    const int nidx = (zc * a.ny + yn) * a.nx + xn;
    if (zn == zc && !a.mask[nidx]) {
      const float behind = *fsi_at<false>(a.fin, a, o, nidx);
      back = 2.f * df * bounced + (1.f - 2.f * df) * behind + 6.f * w * cu;
    }
  }
  // momentum exchange relative to the fluid at rest
  const float hit = bounced + back - 2.f * w;
  const float dfx = hit * (float)(-cxq), dfy = hit * (float)(-cyq);
  fx += dfx;
  fy += dfy;
  mz += (px - a.x_eaf) * dfy - (py - a.y_eaf - a.kinf[z].x) * dfx;
  return back;
}

// Can a cell of this block pull from a wing cell? The sections of layers
// z-1..z+1 lie within `reach` of their elastic axes (lbm_naca.cuh), so a
// block whose sources [x0-1, x0+32] x [y0-1, y0+4] miss those squares sees
// no wing. Blocks on the periodic y edges are always checked cell by cell.
__device__ __forceinline__ bool block_near_wing(const FsiArgs &a, int z) {
  const int xb = (int)blockIdx.x * BX, yb = (int)blockIdx.y * BY;
  if (yb == 0 || yb + BY >= a.ny) return true;
  const float x0 = (float)(xb - 1), x1 = (float)(xb + BX), y0 = (float)(yb - 1), y1 = (float)(yb + BY);
  const int z0 = z > 0 ? z - 1 : 0, z1 = z < a.nz - 1 ? z + 1 : a.nz - 1;
  bool near = false;
  for (int zz = z0; zz <= z1; ++zz) {
    const NacaF &k = a.naca[zz];
    near |= k.reach >= 0.f && x1 >= k.xc0 - k.reach && x0 <= k.xc0 + k.reach && y1 >= k.yc0 - k.reach &&
            y0 <= k.yc0 + k.reach;
  }
  return near;
}

// Resident blocks per SM of the FSI step (0: the compiler's choice, 80-90
// registers; 6, 7 and 8 blocks measured no faster on the 256x128x104 wing).
#ifndef LBM_FSI_MIN_BLOCKS
#define LBM_FSI_MIN_BLOCKS 0
#endif
#if LBM_FSI_MIN_BLOCKS > 0
#define LBM_FSI_BOUNDS __launch_bounds__(BX * BY, LBM_FSI_MIN_BLOCKS)
#else
#define LBM_FSI_BOUNDS __launch_bounds__(BX * BY)
#endif

template <int COLL, bool REPORT, bool FLAT>
__global__ void LBM_FSI_BOUNDS fsi_step_kernel(const __grid_constant__ FsiArgs a) {
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
  const bool near = block_near_wing(a, z);
  float fx = 0.f, fy = 0.f, mz = 0.f;
  if (x < a.nx && y < a.ny) {
    const int idx = (z * a.ny + y) * a.nx + x;
    const bool here = near && a.mask[idx] != 0;
    // source offsets: inflow at x = 0 (no source), zero-gradient outflow at
    // x = nx - 1, periodic y, mirror planes below z = 0 and above z = nz - 1
    const bool inflow = x == 0;
    const int xm = inflow ? 0 : -1, xp = x == a.nx - 1 ? 0 : 1;
    const int ym = y == 0 ? (a.ny - 1) * a.nx : -a.nx, yp = y == a.ny - 1 ? -(a.ny - 1) * a.nx : a.nx;
    const int nxy = a.nx * a.ny;
    const bool zlo = z == 0, zhi = z == a.nz - 1;
    const int zm = zlo ? 0 : -nxy, zp = zhi ? 0 : nxy;
    // every pulled value and, near the wing, every source's mask byte first
    // (independent loads), then the links whose source is in the wing
    float d[Q];
    uint32_t wall = 0;
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      constexpr int mq = dir(cx(q), cy(q), -cz(q));
      const int src = idx + (cx(q) == 1 ? xm : cx(q) == -1 ? xp : 0) + (cy(q) == 1 ? ym : cy(q) == -1 ? yp : 0) +
                      (cz(q) == 1 ? zm : cz(q) == -1 ? zp : 0);
      const bool flip = (cz(q) == 1 && zlo) || (cz(q) == -1 && zhi);
      d[q] = load_l2(fsi_at<FLAT>(a.fin, a, flip ? mq : q, src));
      if (cx(q) == 1 && inflow)
        d[q] = wq(q) * (1.f + 3.f * a.u0 + 4.5f * a.u0 * a.u0 - 1.5f * a.u0 * a.u0);
      // q = 0: a solid cell's own rest population bounces onto itself unchanged
      if (q != 0 && near && a.mask[src]) wall |= 1u << q;
    });
    if (wall) {
      static_for<Q>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        constexpr int o = opp(q);
        if (q != 0 && (wall >> q & 1u)) {
          const int zr = z - cz(q);
          const int zs = zr < 0 ? 0 : (zr > a.nz - 1 ? a.nz - 1 : zr);
          const float bounced = *fsi_at<FLAT>(a.fin, a, o, idx);
          if (here) {
            const float4 k = a.kinf[zs];
            const float px = (float)x - 0.5f * (float)cx(q), py = (float)y - 0.5f * (float)cy(q);
            const float cu = (float)cx(q) * (k.z * (py - a.y_eaf - k.x)) + (float)cy(q) * (k.y - k.z * (px - a.x_eaf));
            d[q] = bounced + 6.f * wq(q) * cu;
          } else {
            d[q] = wetted_link(a, x, y, z, zs, idx, q, o, cx(q), cy(q), cz(q), wq(q), bounced, fx, fy, mz);
          }
        }
      });
    }
    Pairs<float> pr;
    const Moments<float> mo = moments<float, false>(d, !here, pr);
    float post[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) post[q] = d[q];
    collide<float, COLL, false>(post, mo, pr, a.omega_bgk, a.tau0, a.smag_c, a.magic);
    const float t = fmaxf(0.f, ((float)x - a.sponge_start) * a.inv_sponge_len);
    const float sigma = here ? 1.f : a.sponge_strength * t * t;
    // the sponge blend feq(rho_s, u_s) + (1 - sigma)(post - feq(rho, u)); at
    // sigma = 0 it is post up to one rounding, so the cells before the
    // sponge skip it
    if (sigma != 0.f) {
      const float4 k = a.kinf[z];
      const float wx = k.z * ((float)y - a.y_eaf - k.x);
      const float wy = k.y - k.z * ((float)x - a.x_eaf);
      const float rho_s = mo.rho + sigma * (1.f - mo.rho);
      const float usx = here ? wx : mo.ux, usy = here ? wy : mo.uy, usz = here ? 0.f : mo.uz;
      blend_eq<float>(post, eq_base<float>(mo.rho, mo.rho, mo.ux, mo.uy, mo.uz), mo.ux, mo.uy, mo.uz,
                      eq_base<float>(rho_s, rho_s, usx, usy, usz), usx, usy, usz, 1.f - sigma);
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) __stcs(fsi_at<FLAT>(a.fout, a, q, idx), post[q]);
    if (REPORT) {
      a.fld[0][idx] = mo.ux;
      a.fld[1][idx] = mo.uy;
      a.fld[2][idx] = mo.uz;
      a.fld[3][idx] = mo.drho * (1.f / 3.f);
      a.fld[4][idx] = sqrtf(mo.ux * mo.ux + mo.uy * mo.uy + mo.uz * mo.uz);
    }
  }
  // the layer's loads: warp sums, one float64 atomic per warp and component
  // where the warp touched the wing (no block barrier)
  if (near) {
    float v[3] = {fx, fy, mz};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], o);
    }
    if (threadIdx.x == 0)
      for (int c = 0; c < 3; ++c)
        if (v[c] != 0.f) atomicAdd(&a.load[3 * z + c], (double)v[c]);
  }
}

__global__ void fsi_init_kernel(float *f, const uint8_t *mask, int n, float u0) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    float eq[Q];
    feq_val<float, false>(1.f, 1.f, mask[idx] ? 0.f : u0, 0.f, 0.f, eq);
#pragma unroll
    for (int q = 0; q < Q; ++q) f[(size_t)q * n + idx] = eq[q];
  }
}

__global__ void fsi_coarsen_kernel(const float *const *src, float *const *dst, int nx, int ny, int s, int mx, int my,
                                   int m) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < m; idx += gridDim.x * blockDim.x) {
    const int i = idx % mx, j = (idx / mx) % my, k = idx / (mx * my);
    const int from = ((k * s) * ny + j * s) * nx + i * s;
#pragma unroll
    for (int c = 0; c < 5; ++c) dst[c][idx] = src[c][from];
  }
}

}  // namespace lbmf

struct lbm_fsi {
  lbm_fsi_config cfg;
  int64_t n;
  float *f[2] = {nullptr, nullptr};
  int cur = 0;
  uint8_t *mask = nullptr;
  double *kin = nullptr;  // one buffer: KIN doubles, a float4 and a NacaF per layer
  double *load = nullptr;
  unsigned char *kin_host = nullptr;  // pinned staging of kin (uploaded stream-ordered)
  double *load_host = nullptr;        // pinned staging of the loads
  float *fld[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int stride = 1;
  int out_dims[3] = {0, 0, 0};
  float *out[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  float **ptrs = nullptr;
};

namespace {

lbm_status ffail(lbm_status s, const std::string &msg) {
  lbmh::set_last_error(msg);
  return s;
}

#define FCUDA(call)                                                                              \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return ffail(LBM_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

lbm_status fvalidate(const lbm_fsi_config &c) {
  if (c.nx < 2 || c.ny < 2 || c.nz < 1 || (int64_t)c.nx * c.ny * c.nz > (int64_t)INT32_MAX / 19)
    return ffail(LBM_ERR_ARG, "lattice sizes out of range");
  if ((c.ny + lbmk::BY - 1) / lbmk::BY > 65535 || c.nz > 65535) return ffail(LBM_ERR_ARG, "ny/4 and nz must be <= 65535");
  if (c.collision < LBM_BGK || c.collision > LBM_LES) return ffail(LBM_ERR_ARG, "unknown collision model");
  if (!(std::isfinite(c.nu) && c.nu > 0.0)) return ffail(LBM_ERR_ARG, "nu must be finite and > 0");
  if (!(c.chord > 0.0) || !std::isfinite(c.chord)) return ffail(LBM_ERR_ARG, "chord must be > 0");
  const double v[] = {c.cs, c.magic, c.x_ea, c.y_ea, c.ea, c.span, c.u0, c.sponge_start, c.sponge_strength};
  for (double x : v)
    if (!std::isfinite(x)) return ffail(LBM_ERR_ARG, "configuration values must be finite");
  if (!(c.sponge_start < c.nx)) return ffail(LBM_ERR_ARG, "sponge_start must be < nx");
  return LBM_OK;
}

void frelease(lbm_fsi *w) {
  cudaFree(w->f[0]);
  cudaFree(w->f[1]);
  cudaFree(w->mask);
  cudaFree(w->kin);
  cudaFree(w->load);
  cudaFreeHost(w->kin_host);
  cudaFreeHost(w->load_host);
  for (int k = 0; k < 5; ++k) {
    if (w->stride > 1) cudaFree(w->out[k]);
    cudaFree(w->fld[k]);
  }
  cudaFree(w->ptrs);
}

lbmf::FsiArgs fargs(const lbm_fsi *w) {
  const lbm_fsi_config &c = w->cfg;
  lbmf::FsiArgs a{};
  a.mask = w->mask;
  a.kin = w->kin;
  a.kinf = reinterpret_cast<const float4 *>(w->kin + lbmf::KIN * c.nz);
  a.naca = reinterpret_cast<const lbmk::NacaF *>(a.kinf + c.nz);
  a.load = w->load;
  for (int k = 0; k < 5; ++k) a.fld[k] = w->fld[k];
  a.nx = c.nx;
  a.ny = c.ny;
  a.nz = c.nz;
  a.n = (int)w->n;
  a.chord = c.chord;
  a.x_ea = c.x_ea;
  a.y_ea = c.y_ea;
  a.ea = c.ea;
  a.span = c.span;
  a.x_eaf = (float)c.x_ea;
  a.y_eaf = (float)c.y_ea;
  a.u0 = (float)c.u0;
  a.sponge_start = (float)c.sponge_start;
  a.inv_sponge_len = (float)(1.0 / ((double)c.nx - c.sponge_start));
  a.sponge_strength = (float)c.sponge_strength;
  a.omega_bgk = (float)(1.0 / (3.0 * c.nu + 0.5));
  a.tau0 = (float)(3.0 * c.nu + 0.5);
  a.smag_c = (float)(25.456 * c.cs * c.cs);
  a.magic = (float)c.magic;
  return a;
}

size_t kin_bytes(int nz) { return (size_t)nz * (lbmf::KIN * sizeof(double) + sizeof(float4) + sizeof(lbmk::NacaF)); }

// upload the layer kinematics (with cos, sin of each pitch, their float32
// copies and the section prefilter's inputs) and build the mask
lbm_status set_kin(lbm_fsi *w, const double *kin) {
  const lbm_fsi_config &c = w->cfg;
  const int nz = c.nz;
  // the previous upload from the staging buffer has finished once the stream is idle
  FCUDA(cudaStreamSynchronize(0));
  double *k = reinterpret_cast<double *>(w->kin_host);
  float4 *kf = reinterpret_cast<float4 *>(k + lbmf::KIN * nz);
  lbmk::NacaF *nf = reinterpret_cast<lbmk::NacaF *>(kf + nz);
  for (int z = 0; z < nz; ++z) {
    for (int j = 0; j < 4; ++j) k[lbmf::KIN * z + j] = kin[4 * z + j];
    k[lbmf::KIN * z + 4] = std::cos(kin[4 * z + 1]);
    k[lbmf::KIN * z + 5] = std::sin(kin[4 * z + 1]);
    kf[z] = make_float4((float)kin[4 * z], (float)kin[4 * z + 2], (float)kin[4 * z + 3], 0.f);
    nf[z] = lbmk::make_naca_f(c.chord, c.x_ea, c.y_ea + kin[4 * z], c.ea, k[lbmf::KIN * z + 4],
                              k[lbmf::KIN * z + 5]);
    if (!((double)z + 0.5 < c.span)) nf[z].reach = -1.f;  // past the tip: no section
  }
  FCUDA(cudaMemcpyAsync(w->kin, w->kin_host, kin_bytes(nz), cudaMemcpyHostToDevice, 0));
  lbmf::fsi_mask_kernel<<<lbmk::cell_grid(w->n), 256>>>(fargs(w), w->mask);
  FCUDA(cudaGetLastError());
  return LBM_OK;
}

template <int COLL>
void launch_fsi(const lbm_fsi *w, const lbmf::FsiArgs &a, bool report) {
  const dim3 block(lbmk::BX, lbmk::BY);
  const dim3 grid((w->cfg.nx + lbmk::BX - 1) / lbmk::BX, (w->cfg.ny + lbmk::BY - 1) / lbmk::BY, w->cfg.nz);
  if (19 * (int64_t)w->n <= (int64_t)UINT32_MAX) {
    if (report) lbmf::fsi_step_kernel<COLL, true, true><<<grid, block>>>(a);
    else lbmf::fsi_step_kernel<COLL, false, true><<<grid, block>>>(a);
  } else {
    if (report) lbmf::fsi_step_kernel<COLL, true, false><<<grid, block>>>(a);
    else lbmf::fsi_step_kernel<COLL, false, false><<<grid, block>>>(a);
  }
}

lbm_status fset_ptrs(lbm_fsi *w) {
  float *h[10];
  for (int k = 0; k < 5; ++k) {
    h[k] = w->fld[k];
    h[5 + k] = w->out[k];
  }
  FCUDA(cudaMemcpy(w->ptrs, h, sizeof(h), cudaMemcpyHostToDevice));
  return LBM_OK;
}

}  // namespace

extern "C" {

lbm_status lbm_fsi_create(const lbm_fsi_config *cfg, lbm_fsi **out) {
  if (!cfg || !out) return ffail(LBM_ERR_ARG, "null argument");
  *out = nullptr;
  lbm_status st = fvalidate(*cfg);
  if (st != LBM_OK) return st;
  FCUDA(cudaSetDevice(cfg->device));
  lbm_fsi *w = new (std::nothrow) lbm_fsi();
  if (!w) return ffail(LBM_ERR_ARG, "out of host memory");
  w->cfg = *cfg;
  w->n = (int64_t)cfg->nx * cfg->ny * cfg->nz;
  w->out_dims[0] = cfg->nx;
  w->out_dims[1] = cfg->ny;
  w->out_dims[2] = cfg->nz;
  const size_t fb = (size_t)19 * w->n * sizeof(float);
  cudaError_t e = cudaMalloc(&w->f[0], fb);
  if (e == cudaSuccess) e = cudaMalloc(&w->f[1], fb);
  if (e == cudaSuccess) e = cudaMalloc(&w->mask, (size_t)w->n);
  if (e == cudaSuccess) e = cudaMalloc(&w->kin, kin_bytes(cfg->nz));
  if (e == cudaSuccess) e = cudaMallocHost(&w->kin_host, kin_bytes(cfg->nz));
  if (e == cudaSuccess) e = cudaMallocHost(&w->load_host, (size_t)3 * cfg->nz * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(w->kin, 0, kin_bytes(cfg->nz));
  if (e == cudaSuccess) e = cudaMalloc(&w->load, (size_t)3 * cfg->nz * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&w->ptrs, 10 * sizeof(float *));
  for (int k = 0; k < 5 && e == cudaSuccess; ++k) {
    e = cudaMallocManaged(&w->fld[k], (size_t)w->n * sizeof(float), cudaMemAttachGlobal);
    if (e == cudaSuccess) e = cudaMemset(w->fld[k], 0, (size_t)w->n * sizeof(float));
    w->out[k] = w->fld[k];
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    frelease(w);
    delete w;
    return ffail(LBM_ERR_CUDA, std::string("lbm_fsi_create: ") + cudaGetErrorString(e));
  }
  *out = w;
  return LBM_OK;
}

lbm_status lbm_fsi_destroy(lbm_fsi *w) {
  if (!w) return LBM_OK;
  cudaSetDevice(w->cfg.device);
  cudaDeviceSynchronize();
  frelease(w);
  delete w;
  return LBM_OK;
}

lbm_status lbm_fsi_init(lbm_fsi *w, const double *kin) {
  if (!w || !kin) return ffail(LBM_ERR_ARG, "null argument");
  FCUDA(cudaSetDevice(w->cfg.device));
  lbm_status st = set_kin(w, kin);
  if (st != LBM_OK) return st;
  w->cur = 0;
  lbmf::fsi_init_kernel<<<lbmk::cell_grid(w->n), 256>>>(w->f[0], w->mask, (int)w->n, (float)w->cfg.u0);
  FCUDA(cudaGetLastError());
  return LBM_OK;
}

lbm_status lbm_fsi_step(lbm_fsi *w, int32_t report, const double *kin, double *load) {
  lbmh::Range range_("lbm_fsi_step");
  if (!w || !kin || !load) return ffail(LBM_ERR_ARG, "null argument");
  FCUDA(cudaSetDevice(w->cfg.device));
  lbm_status st = set_kin(w, kin);
  if (st != LBM_OK) return st;
  lbmf::FsiArgs a = fargs(w);
  a.fin = w->f[w->cur];
  a.fout = w->f[1 - w->cur];
  FCUDA(cudaMemsetAsync(w->load, 0, (size_t)3 * w->cfg.nz * sizeof(double)));
  switch (w->cfg.collision) {
    case LBM_BGK: launch_fsi<lbmk::COLL_BGK>(w, a, report != 0); break;
    case LBM_TRT: launch_fsi<lbmk::COLL_TRT>(w, a, report != 0); break;
    default: launch_fsi<lbmk::COLL_LES>(w, a, report != 0); break;
  }
  FCUDA(cudaGetLastError());
  const size_t lb = (size_t)3 * w->cfg.nz * sizeof(double);
  FCUDA(cudaMemcpyAsync(w->load_host, w->load, lb, cudaMemcpyDeviceToHost, 0));
  FCUDA(cudaStreamSynchronize(0));
  std::memcpy(load, w->load_host, lb);
  w->cur ^= 1;
  return LBM_OK;
}

lbm_status lbm_fsi_set_physics(lbm_fsi *w, int32_t collision, double nu) {
  if (!w) return ffail(LBM_ERR_ARG, "null argument");
  lbm_fsi_config c = w->cfg;
  c.collision = collision;
  c.nu = nu;
  lbm_status st = fvalidate(c);
  if (st != LBM_OK) return st;
  w->cfg = c;
  return LBM_OK;
}

lbm_status lbm_fsi_field(lbm_fsi *w, int32_t id, float **ptr) {
  if (!w || !ptr) return ffail(LBM_ERR_ARG, "null argument");
  if (id < 0 || id >= 5) return ffail(LBM_ERR_ARG, "field id out of range (ux, uy, uz, p, vmag)");
  *ptr = w->fld[id];
  return LBM_OK;
}

lbm_status lbm_fsi_populations(lbm_fsi *w, float *host, int32_t set) {
  if (!w || !host) return ffail(LBM_ERR_ARG, "null argument");
  FCUDA(cudaSetDevice(w->cfg.device));
  const size_t fb = (size_t)19 * w->n * sizeof(float);
  if (set) FCUDA(cudaMemcpy(w->f[w->cur], host, fb, cudaMemcpyHostToDevice));
  else FCUDA(cudaMemcpy(host, w->f[w->cur], fb, cudaMemcpyDeviceToHost));
  return LBM_OK;
}

lbm_status lbm_fsi_mask(lbm_fsi *w, const double *kin, uint8_t *host) {
  if (!w || !kin || !host) return ffail(LBM_ERR_ARG, "null argument");
  FCUDA(cudaSetDevice(w->cfg.device));
  lbm_status st = set_kin(w, kin);
  if (st != LBM_OK) return st;
  FCUDA(cudaMemcpy(host, w->mask, (size_t)w->n, cudaMemcpyDeviceToHost));
  return LBM_OK;
}

lbm_status lbm_fsi_set_output_stride(lbm_fsi *w, int32_t stride) {
  if (!w) return ffail(LBM_ERR_ARG, "null argument");
  if (stride < 1) return ffail(LBM_ERR_ARG, "stride must be >= 1");
  FCUDA(cudaSetDevice(w->cfg.device));
  FCUDA(cudaDeviceSynchronize());
  if (w->stride > 1)
    for (int k = 0; k < 5; ++k) cudaFree(w->out[k]);
  const int dims[3] = {w->cfg.nx, w->cfg.ny, w->cfg.nz};
  size_t m = 1;
  for (int k = 0; k < 3; ++k) {
    w->out_dims[k] = (dims[k] + stride - 1) / stride;
    m *= (size_t)w->out_dims[k];
  }
  w->stride = stride;
  for (int k = 0; k < 5; ++k) {
    if (stride == 1) {
      w->out[k] = w->fld[k];
      continue;
    }
    FCUDA(cudaMallocManaged(&w->out[k], m * sizeof(float), cudaMemAttachGlobal));
    FCUDA(cudaMemset(w->out[k], 0, m * sizeof(float)));
  }
  return fset_ptrs(w);
}

lbm_status lbm_fsi_output(lbm_fsi *w, int32_t id, float **ptr, int64_t *count) {
  if (!w || !ptr || !count) return ffail(LBM_ERR_ARG, "null argument");
  if (id < 0 || id >= 5) return ffail(LBM_ERR_ARG, "output id out of range (ux, uy, uz, p, vmag)");
  *ptr = w->out[id];
  *count = (int64_t)w->out_dims[0] * w->out_dims[1] * w->out_dims[2];
  return LBM_OK;
}

lbm_status lbm_fsi_update_output(lbm_fsi *w) {
  if (!w) return ffail(LBM_ERR_ARG, "null argument");
  if (w->stride <= 1) return LBM_OK;
  FCUDA(cudaSetDevice(w->cfg.device));
  const int m = w->out_dims[0] * w->out_dims[1] * w->out_dims[2];
  lbmf::fsi_coarsen_kernel<<<lbmk::cell_grid(m), 256>>>(w->ptrs, w->ptrs + 5, w->cfg.nx, w->cfg.ny, w->stride,
                                                        w->out_dims[0], w->out_dims[1], m);
  FCUDA(cudaGetLastError());
  return LBM_OK;
}

}  // extern "C"
