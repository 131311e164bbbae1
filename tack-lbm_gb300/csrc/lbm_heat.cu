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
};

template <bool REPORT>
__global__ void __launch_bounds__(256) heat_kernel(const __grid_constant__ HeatArgs h) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < h.n; idx += gridDim.x * blockDim.x) {
    const int x = idx % h.nx, y = (idx / h.nx) % h.ny, z = idx / (h.nx * h.ny);
    const bool here = solid(h.geo, x, y, z);
    const float fluid = here ? 0.f : 1.f;
    float g[7], temp = 0.f;
    int src[7];
    static_for<7>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      int xs = x - cx7(q), ys = y - cy7(q), zs = z - cz7(q);
      xs += xs < 0 ? h.nx : 0;
      xs -= xs >= h.nx ? h.nx : 0;
      ys += ys < 0 ? h.ny : 0;
      ys -= ys >= h.ny ? h.ny : 0;
      zs += zs < 0 ? h.nz : 0;
      zs -= zs >= h.nz ? h.nz : 0;
      const int nidx = (zs * h.ny + ys) * h.nx + xs;
      src[q] = nidx;
      const float pulled = load_l2(h.g_in + (size_t)q * h.n + nidx);
      float val = pulled;
      if (q != 0 && solid(h.geo, xs, ys, zs)) {
        const float bounced = h.g_in[(size_t)opp7(q) * h.n + idx];
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
      __stcs(h.g_out + (size_t)q * h.n + idx, es + keep * (post - eq));
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
  const int grid = lbmk::cell_grid(c.n);
  if (report) {
    cudaMemsetAsync(c.heat_fld[LBM_Q_SOLID], 0, (size_t)c.n * sizeof(float), st);
    lbmk::heat_kernel<true><<<grid, 256, 0, st>>>(h);
  } else {
    lbmk::heat_kernel<false><<<grid, 256, 0, st>>>(h);
  }
  return cudaGetLastError();
}

}  // namespace lbmh
