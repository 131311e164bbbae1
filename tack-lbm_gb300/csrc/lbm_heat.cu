// lbm_heat.cu - the D3Q7 temperature block of the step (lbm.py:457-492).
//
// Temperature is advected and diffused with a D3Q7 lattice (c_s^2 = 1/4,
// lbm.py:20-25) on A/B buffers g[q*n + idx] in FP32. It runs as its own
// launch right after the flow step on the same stream. The flow kernel leaves
// the moments it computed for every fluid cell, (ux, uy, uz, tau), in `aux`,
// so this kernel needs no second pass over the 19 flow populations.
//
// Per cell, as the reference step does it:
//   * streaming from the periodic neighbour, with the sink faces holding the
//     solid's temperature by anti-bounce-back and the duct walls adiabatic by
//     bounce-back: g_q = p + wall (b (1 - 2 hot) + hot 2 w_q T_s - p);
//   * diffusivity alpha + max(0, (tau - 1/2)/3 - nu)/Pr_t with Pr_t = 0.85
//     (lbm.py:299-301), relaxation 1/(4 alpha + 1/2);
//   * the sponge blend of the flow (the same sigma and target velocity), with
//     the temperature relaxed toward 0 in the sponge and inside solids;
//   * report steps write the temperature field (the solid's own temperature
//     in solid cells) and add each fluid cell's temperature to every sink
//     voxel it faces (q_solid, one atomic add per wetted face, lbm.py:484-492).
#include <cuda_runtime.h>

#include "lbm_device.cuh"
#include "lbm_host.h"

namespace lbmk {

// D3Q7 (lbm.py:20-25)
__host__ __device__ constexpr int cx7(int q) { return q == 1 ? 1 : q == 2 ? -1 : 0; }
__host__ __device__ constexpr int cy7(int q) { return q == 3 ? 1 : q == 4 ? -1 : 0; }
__host__ __device__ constexpr int cz7(int q) { return q == 5 ? 1 : q == 6 ? -1 : 0; }
__host__ __device__ constexpr int opp7(int q) { return q == 0 ? 0 : (q & 1 ? q + 1 : q - 1); }
__host__ __device__ constexpr float w7(int q) { return q == 0 ? 0.25f : 0.125f; }
constexpr float PR_T = 0.85f;  // turbulent Prandtl number (lbm.py:285)

struct HeatArgs {
  const float *g_in;
  float *g_out;
  const float4 *aux;
  const float *t_solid;
  float *q_solid, *temp;
  Geo geo;
  int nx, ny, nz, n;
  float u0, sponge_start, inv_sponge_len, sponge_strength;
  float alpha, nu, tau0;
  // the flow step's link masks (bit q, q = 1..6: the source x - c_q is solid;
  // bit 19: the cell is solid) over the obstacle's reach box; used when y and
  // z are periodic, where the flow's sources are the temperature's sources
  const uint32_t *masks;
  int reach_lo[3], reach_hi[3], reach_any, use_masks;
};

// first link-mask word of the 32-cell row segment at x0, or -1 outside the reach box
__device__ __forceinline__ int heat_mask_slot(const HeatArgs &h, int x0, int y, int z) {
  if (!h.reach_any || x0 + BX - 1 < h.reach_lo[0] || x0 > h.reach_hi[0] || y < h.reach_lo[1] ||
      y > h.reach_hi[1] || z < h.reach_lo[2] || z > h.reach_hi[2])
    return -1;
  const int w0 = h.reach_lo[0] / BX, nw = h.reach_hi[0] / BX - w0 + 1;
  const int nyr = h.reach_hi[1] - h.reach_lo[1] + 1;
  return (((z - h.reach_lo[2]) * nyr + (y - h.reach_lo[1])) * nw + (x0 / BX - w0)) * BX;
}

// Slot q of cell e in an A/B temperature buffer: FLAT (7 n < 2^32) forms a
// 32-bit element offset from the base, else a 64-bit one.
template <bool FLAT, typename P>
__device__ __forceinline__ P *heat_at(P *g, const HeatArgs &h, int q, int e) {
  if (FLAT) return g + (uint32_t)((uint32_t)q * (uint32_t)h.n + (uint32_t)e);
  return g + (size_t)q * h.n + e;
}

// One cell per thread; a warp is a 32-cell row segment (block 32 x 8). The
// sources come from six per-cell neighbour offsets; their coordinates are
// formed only where a wall or sink test needs them.
template <bool REPORT, bool FLAT>
__global__ void __launch_bounds__(256) heat_kernel(const __grid_constant__ HeatArgs h) {
  const int x0 = (int)blockIdx.x * BX, x = x0 + (int)threadIdx.x;
  const int y = (int)blockIdx.y * blockDim.y + (int)threadIdx.y, z = (int)blockIdx.z;
  if (y >= h.ny) return;  // whole warps: blockDim.x is 32
  uint32_t m = 0;
  if (h.use_masks) {
    const int ms = heat_mask_slot(h, x0, y, z);
    m = ms >= 0 ? h.masks[ms + (int)threadIdx.x] : 0u;
  }
  if (x >= h.nx) return;
  const int idx = (z * h.ny + y) * h.nx + x;
  const bool here = h.use_masks ? (m & MASK_SOLID) != 0 : solid(h.geo, x, y, z);
  const float fluid = here ? 0.f : 1.f;
  float g[7], temp = 0.f;
  int src[7];
  const int nxy = h.nx * h.ny;
  const int dxm = x == 0 ? h.nx - 1 : -1, dxp = x == h.nx - 1 ? 1 - h.nx : 1;
  const int dym = y == 0 ? nxy - h.nx : -h.nx, dyp = y == h.ny - 1 ? h.nx - nxy : h.nx;
  const int dzm = z == 0 ? (h.nz - 1) * nxy : -nxy, dzp = z == h.nz - 1 ? -(h.nz - 1) * nxy : nxy;
  static_for<7>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    // the source x - c_q, periodic in all three axes
    const int nidx = idx + (cx7(q) == 1 ? dxm : cx7(q) == -1 ? dxp : 0) +
                     (cy7(q) == 1 ? dym : cy7(q) == -1 ? dyp : 0) + (cz7(q) == 1 ? dzm : cz7(q) == -1 ? dzp : 0);
    auto coords = [&](int &xs, int &ys, int &zs) {
      xs = x - cx7(q);
      ys = y - cy7(q);
      zs = z - cz7(q);
      xs += xs < 0 ? h.nx : 0;
      xs -= xs >= h.nx ? h.nx : 0;
      ys += ys < 0 ? h.ny : 0;
      ys -= ys >= h.ny ? h.ny : 0;
      zs += zs < 0 ? h.nz : 0;
      zs -= zs >= h.nz ? h.nz : 0;
    };
    src[q] = nidx;
    const float pulled = load_l2(heat_at<FLAT>(h.g_in, h, q, nidx));
    float val = pulled;
    // D3Q7 direction q (1..6) is D3Q19 direction q: the same link-mask bit
    bool wall = false;
    if (q != 0) {
      if (h.use_masks) {
        wall = ((m >> q) & 1u) != 0;
      } else {
        int xs, ys, zs;
        coords(xs, ys, zs);
        wall = solid(h.geo, xs, ys, zs);
      }
    }
    if (wall) {
      int xs, ys, zs;
      coords(xs, ys, zs);
      const float bounced = *heat_at<FLAT>(h.g_in, h, opp7(q), idx);
      val = sink(h.geo, xs, ys, zs) ? -bounced + 2.0f * w7(q) * h.t_solid[nidx] : bounced;
    }
    g[q] = val;
    temp += val;
  });
  float ux = 0.f, uy = 0.f, uz = 0.f, tau = h.tau0;
  if (!here) {
    const float4 a = __ldcs(h.aux + idx);  // read once, after the flow step wrote it
    ux = a.x;
    uy = a.y;
    uz = a.z;
    tau = a.w;
  }
  const float t = fmaxf(0.f, ((float)x - h.sponge_start) * h.inv_sponge_len);
  const float sigma = here ? 1.f : h.sponge_strength * t * t;
  const float keep = 1.f - sigma;
  const float usx = ux + sigma * (h.u0 * fluid - ux), usy = keep * uy, usz = keep * uz;
  const float alpha = h.alpha + fmaxf(0.f, (tau - 0.5f) * (1.f / 3.f) - h.nu) * (1.f / PR_T);
  const float om = 1.f / (4.f * alpha + 0.5f);
  const float temp_s = keep * temp;
  static_for<7>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    const float eq = w7(q) * temp * (1.f + 4.f * ((float)cx7(q) * ux + (float)cy7(q) * uy + (float)cz7(q) * uz));
    const float post = g[q] - om * (g[q] - eq);
    const float es = w7(q) * temp_s * (1.f + 4.f * ((float)cx7(q) * usx + (float)cy7(q) * usy + (float)cz7(q) * usz));
    __stcs(heat_at<FLAT>(h.g_out, h, q, idx), es + keep * (post - eq));
  });
  if (REPORT) {
    h.temp[idx] = here ? h.t_solid[idx] : temp;
    if (!here) {
      static_for<7>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        if (q != 0) {
          const int s = src[q];
          const int xs = s % h.nx, ys = (s / h.nx) % h.ny, zs = s / (h.nx * h.ny);
          if (sink(h.geo, xs, ys, zs)) atomicAdd(&h.q_solid[s], temp);
        }
      });
    }
  }
}

}  // namespace lbmk

namespace lbmh {

cudaError_t launch_heat(const Ctx &c, bool report, cudaStream_t st) {
  lbmk::HeatArgs h{};
  const lbm_config &g = c.cfg;
  h.g_in = c.g[c.g_cur];
  h.g_out = c.g[1 - c.g_cur];
  h.aux = c.aux;
  h.t_solid = c.heat_fld[LBM_T_SOLID];
  h.q_solid = c.heat_fld[LBM_Q_SOLID];
  h.temp = c.heat_fld[LBM_TEMP];
  h.geo = lbmk::make_geo(g);
  h.nx = g.nx;
  h.ny = g.ny;
  h.nz = g.nz;
  h.n = (int)c.n;
  h.u0 = (float)g.u0;
  h.sponge_start = (float)g.sponge_start;
  h.inv_sponge_len = (float)(1.0 / ((double)g.nx - g.sponge_start));
  h.sponge_strength = (float)g.sponge_strength;
  h.alpha = (float)g.alpha;
  h.nu = (float)g.heat_nu;
  h.tau0 = (float)(3.0 * g.nu + 0.5);
  h.masks = c.wmasks;
  for (int k = 0; k < 3; ++k) {
    h.reach_lo[k] = c.reach_lo[k];
    h.reach_hi[k] = c.reach_hi[k];
  }
  h.reach_any = c.reach_any;
  h.use_masks = g.lateral == LBM_PERIODIC && g.vertical == LBM_PERIODIC && (!c.reach_any || c.wmasks) ? 1 : 0;
  const dim3 block(lbmk::BX, 8);
  const dim3 grid((g.nx + lbmk::BX - 1) / lbmk::BX, (g.ny + 7) / 8, g.nz);
  const bool flat = 7 * c.n <= (int64_t)UINT32_MAX;
  if (report) {
    cudaMemsetAsync(c.heat_fld[LBM_Q_SOLID], 0, (size_t)c.n * sizeof(float), st);
    if (flat) lbmk::heat_kernel<true, true><<<grid, block, 0, st>>>(h);
    else lbmk::heat_kernel<true, false><<<grid, block, 0, st>>>(h);
  } else {
    if (flat) lbmk::heat_kernel<false, true><<<grid, block, 0, st>>>(h);
    else lbmk::heat_kernel<false, false><<<grid, block, 0, st>>>(h);
  }
  return cudaGetLastError();
}

}  // namespace lbmh
