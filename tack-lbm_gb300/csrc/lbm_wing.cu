// lbm_wing.cu - the pitch-plunge wing step (tack-lbm flutter.py:20-130) and its C ABI.
//
// A rigid NACA 0012 section spanning z moves with the plunge h and pitch alpha
// about its elastic axis; the structure (integrated on the host) and the
// fluid exchange data every step. Per step:
//   * wing_mask_kernel evaluates the section test (flutter.py:30-42) once per
//     cell into a byte mask with float64 results (a float32 prefilter decides
//     the cells away from the outline, lbm_naca.cuh), so the mask is exact and
//     the step kernel's 19 source tests are byte loads (mostly L1 hits);
//   * wing_step_kernel (float32, A/B buffers f[q*n + idx], one thread per
//     cell, periodic in x, y and z) pulls the populations, applies halfway
//     bounce-back on the moving wall with the term 6 w_q c_q.u_wall at the link
//     midpoint, collects the momentum-exchange force and its moment about the
//     displaced elastic axis, collides (the solver's BGK / TRT / LES), blends
//     the sponge and relaxes solid cells to equilibrium at the wall velocity
//     (flutter.py:116-126), and on report steps writes ux, uy, uz, p, vmag.
//   The force and moment are reduced per block with warp shuffles and added
//   to three float64 totals, one atomic per block and component (the
//   reference adds every wetted cell's values with float atomics).
#include <cuda_runtime.h>

#include <cmath>
#include <new>
#include <string>
#include <vector>

#include "lbm_device.cuh"
#include "lbm_host.h"
#include "lbm_naca.cuh"

namespace lbmw {

using namespace lbmk;

struct WingArgs {
  const float *fin;
  float *fout;
  const uint8_t *mask;
  double *load;  // fx, fy, mz
  float *fld[5];
  int nx, ny, nz, n;
  float x_ea, y_ea, h, dh, da;
  float u0, sponge_start, inv_sponge_len, sponge_strength;
  float omega_bgk, tau0, smag_c, magic;
};

// the section test of flutter.py:30-42 in float64, after the float32 prefilter
__global__ void wing_mask_kernel(uint8_t *mask, int nx, int ny, int n, NacaF nf, double chord, double x_ea,
                                 double y_ea, double ea, double h, double ca, double sa) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const int x = idx % nx, y = (idx / nx) % ny;
    const int r = naca_prefilter(nf, (float)x, (float)y);
    if (r != 0) {
      mask[idx] = r > 0 ? 1 : 0;
      continue;
    }
    const double dx = (double)x - x_ea, dy = (double)y - (y_ea + h);
    const double s = dx * ca - dy * sa, t = dx * sa + dy * ca;
    const double xc = s / chord + ea;
    const double c = fmin(fmax(xc, 0.0), 1.0);
    const double half = 0.6 * chord * (0.2969 * sqrt(c) - 0.1260 * c - 0.3516 * c * c + 0.2843 * c * c * c -
                                       0.1036 * c * c * c * c);
    mask[idx] = (xc >= 0.0 && xc <= 1.0 && fabs(t) < half) ? 1 : 0;
  }
}

template <int COLL, bool REPORT>
__global__ void __launch_bounds__(BX * BY) wing_step_kernel(const __grid_constant__ WingArgs a) {
  const int x = blockIdx.x * BX + threadIdx.x, y = blockIdx.y * BY + threadIdx.y, z = blockIdx.z;
  float fx = 0.f, fy = 0.f, mz = 0.f;
  if (x < a.nx && y < a.ny) {
    const int idx = (z * a.ny + y) * a.nx + x;
    const bool here = a.mask[idx] != 0;
    const int xm = x == 0 ? a.nx - 1 : -1, xp = x == a.nx - 1 ? 1 - a.nx : 1;
    const int ym = y == 0 ? (a.ny - 1) * a.nx : -a.nx, yp = y == a.ny - 1 ? -(a.ny - 1) * a.nx : a.nx;
    const int nxy = a.nx * a.ny;
    const int zm = z == 0 ? (a.nz - 1) * nxy : -nxy, zp = z == a.nz - 1 ? -(a.nz - 1) * nxy : nxy;
    // every pulled value and every source's mask byte first (independent
    // loads), then the links whose source is in the wing
    float d[Q];
    uint32_t wall = 0;
    static_for<Q>([&](auto qc) {
      constexpr int q = decltype(qc)::value;
      // source x - c_q
      const int src = idx + (cx(q) == 1 ? xm : cx(q) == -1 ? xp : 0) + (cy(q) == 1 ? ym : cy(q) == -1 ? yp : 0) +
                      (cz(q) == 1 ? zm : cz(q) == -1 ? zp : 0);
      d[q] = load_l2(a.fin + (size_t)q * a.n + src);
      if (q != 0 && a.mask[src]) wall |= 1u << q;
    });
    if (wall) {
      static_for<Q>([&](auto qc) {
        constexpr int q = decltype(qc)::value;
        if (q != 0 && (wall >> q & 1u)) {
          const float bounced = a.fin[(size_t)opp(q) * a.n + idx];
          const float px = (float)x - 0.5f * (float)cx(q), py = (float)y - 0.5f * (float)cy(q);
          const float wx = a.da * (py - a.y_ea - a.h), wy = a.dh - a.da * (px - a.x_ea);
          const float back = bounced + 6.f * wq(q) * ((float)cx(q) * wx + (float)cy(q) * wy);
          d[q] = back;
          if (!here) {
            const float hit = bounced + back;
            const float dfx = hit * (float)(-cx(q)), dfy = hit * (float)(-cy(q));
            fx += dfx;
            fy += dfy;
            mz += (px - a.x_ea) * dfy - (py - a.y_ea - a.h) * dfx;
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
    // the sponge blend; at sigma = 0 it is post up to one rounding
    if (sigma != 0.f) {
      const float wx = a.da * ((float)y - a.y_ea - a.h), wy = a.dh - a.da * ((float)x - a.x_ea);
      const float tx = here ? wx : a.u0, ty = here ? wy : 0.f;
      const float rho_s = mo.rho + sigma * (1.f - mo.rho);
      const float usx = mo.ux + sigma * (tx - mo.ux), usy = mo.uy + sigma * (ty - mo.uy),
                  usz = (1.f - sigma) * mo.uz;
      blend_eq<float>(post, eq_base<float>(mo.rho, mo.rho, mo.ux, mo.uy, mo.uz), mo.ux, mo.uy, mo.uz,
                      eq_base<float>(rho_s, rho_s, usx, usy, usz), usx, usy, usz, 1.f - sigma);
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) __stcs(a.fout + (size_t)q * a.n + idx, post[q]);
    if (REPORT) {
      a.fld[0][idx] = mo.ux;
      a.fld[1][idx] = mo.uy;
      a.fld[2][idx] = mo.uz;
      a.fld[3][idx] = mo.drho * (1.f / 3.f);
      a.fld[4][idx] = sqrtf(mo.ux * mo.ux + mo.uy * mo.uy + mo.uz * mo.uz);
    }
  }
  // block sums of the force and moment, one float64 atomic per component
  __shared__ float red[BY][3];
  float v[3] = {fx, fy, mz};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) red[threadIdx.y][k] = v[k];
  __syncthreads();
  if (threadIdx.y == 0 && threadIdx.x < 3) {
    float s = 0.f;
    for (int w = 0; w < BY; ++w) s += red[w][threadIdx.x];
    if (s != 0.f) atomicAdd(&a.load[threadIdx.x], (double)s);
  }
}

__global__ void wing_init_kernel(float *f, const uint8_t *mask, int n, float u0) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    float eq[Q];
    feq_val<float, false>(1.f, 1.f, mask[idx] ? 0.f : u0, 0.f, 0.f, eq);
#pragma unroll
    for (int q = 0; q < Q; ++q) f[(size_t)q * n + idx] = eq[q];
  }
}

__global__ void wing_coarsen_kernel(const float *const *src, float *const *dst, int nx, int ny, int s, int mx,
                                    int my, int m) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < m; idx += gridDim.x * blockDim.x) {
    const int i = idx % mx, j = (idx / mx) % my, k = idx / (mx * my);
    const int from = ((k * s) * ny + j * s) * nx + i * s;
#pragma unroll
    for (int f = 0; f < 5; ++f) dst[f][idx] = src[f][from];
  }
}

}  // namespace lbmw

struct lbm_wing {
  lbm_wing_config cfg;
  int64_t n;
  float *f[2] = {nullptr, nullptr};
  int cur = 0;
  uint8_t *mask = nullptr;
  double *load = nullptr;
  float *fld[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int stride = 1;
  int out_dims[3] = {0, 0, 0};
  float *out[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  float **ptrs = nullptr;  // device copies of fld and out for the coarsen kernel
};

namespace {

lbm_status wfail(lbm_status s, const std::string &msg) {
  lbmh::set_last_error(msg);
  return s;
}

#define WCUDA(call)                                                                              \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return wfail(LBM_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

lbm_status wvalidate(const lbm_wing_config &c) {
  if (c.nx < 2 || c.ny < 2 || c.nz < 1 || (int64_t)c.nx * c.ny * c.nz > (int64_t)INT32_MAX / 19)
    return wfail(LBM_ERR_ARG, "lattice sizes out of range");
  if ((c.ny + lbmk::BY - 1) / lbmk::BY > 65535 || c.nz > 65535) return wfail(LBM_ERR_ARG, "ny/4 and nz must be <= 65535");
  if (c.collision < LBM_BGK || c.collision > LBM_LES) return wfail(LBM_ERR_ARG, "unknown collision model");
  if (!(std::isfinite(c.nu) && c.nu > 0.0)) return wfail(LBM_ERR_ARG, "nu must be finite and > 0");
  if (!(c.chord > 0.0) || !std::isfinite(c.chord)) return wfail(LBM_ERR_ARG, "chord must be > 0");
  const double v[] = {c.cs, c.magic, c.x_ea, c.y_ea, c.ea, c.u0, c.sponge_start, c.sponge_strength};
  for (double x : v)
    if (!std::isfinite(x)) return wfail(LBM_ERR_ARG, "configuration values must be finite");
  if (!(c.sponge_start < c.nx)) return wfail(LBM_ERR_ARG, "sponge_start must be < nx");
  return LBM_OK;
}

void wrelease(lbm_wing *w) {
  cudaFree(w->f[0]);
  cudaFree(w->f[1]);
  cudaFree(w->mask);
  cudaFree(w->load);
  for (int k = 0; k < 5; ++k) {
    if (w->stride > 1) cudaFree(w->out[k]);
    cudaFree(w->fld[k]);
  }
  cudaFree(w->ptrs);
}

lbm_status build_mask(lbm_wing *w, const double st[4]) {
  const lbm_wing_config &c = w->cfg;
  const double ca = std::cos(st[1]), sa = std::sin(st[1]);
  const lbmk::NacaF nf = lbmk::make_naca_f(c.chord, c.x_ea, c.y_ea + st[0], c.ea, ca, sa);
  lbmw::wing_mask_kernel<<<lbmk::cell_grid(w->n), 256>>>(w->mask, c.nx, c.ny, (int)w->n, nf, c.chord, c.x_ea,
                                                         c.y_ea, c.ea, st[0], ca, sa);
  WCUDA(cudaGetLastError());
  return LBM_OK;
}

template <int COLL>
void launch_wing(const lbm_wing *w, const lbmw::WingArgs &a, bool report) {
  const dim3 block(lbmk::BX, lbmk::BY);
  const dim3 grid((w->cfg.nx + lbmk::BX - 1) / lbmk::BX, (w->cfg.ny + lbmk::BY - 1) / lbmk::BY, w->cfg.nz);
  if (report) lbmw::wing_step_kernel<COLL, true><<<grid, block>>>(a);
  else lbmw::wing_step_kernel<COLL, false><<<grid, block>>>(a);
}

lbm_status set_ptrs(lbm_wing *w) {
  float *h[10];
  for (int k = 0; k < 5; ++k) {
    h[k] = w->fld[k];
    h[5 + k] = w->out[k];
  }
  WCUDA(cudaMemcpy(w->ptrs, h, sizeof(h), cudaMemcpyHostToDevice));
  return LBM_OK;
}

}  // namespace

extern "C" {

lbm_status lbm_wing_create(const lbm_wing_config *cfg, lbm_wing **out) {
  if (!cfg || !out) return wfail(LBM_ERR_ARG, "null argument");
  *out = nullptr;
  lbm_status st = wvalidate(*cfg);
  if (st != LBM_OK) return st;
  WCUDA(cudaSetDevice(cfg->device));
  lbm_wing *w = new (std::nothrow) lbm_wing();
  if (!w) return wfail(LBM_ERR_ARG, "out of host memory");
  w->cfg = *cfg;
  w->n = (int64_t)cfg->nx * cfg->ny * cfg->nz;
  w->out_dims[0] = cfg->nx;
  w->out_dims[1] = cfg->ny;
  w->out_dims[2] = cfg->nz;
  const size_t fb = (size_t)19 * w->n * sizeof(float);
  cudaError_t e = cudaMalloc(&w->f[0], fb);
  if (e == cudaSuccess) e = cudaMalloc(&w->f[1], fb);
  if (e == cudaSuccess) e = cudaMalloc(&w->mask, (size_t)w->n);
  if (e == cudaSuccess) e = cudaMalloc(&w->load, 3 * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&w->ptrs, 10 * sizeof(float *));
  for (int k = 0; k < 5 && e == cudaSuccess; ++k) {
    e = cudaMallocManaged(&w->fld[k], (size_t)w->n * sizeof(float), cudaMemAttachGlobal);
    if (e == cudaSuccess) e = cudaMemset(w->fld[k], 0, (size_t)w->n * sizeof(float));
    w->out[k] = w->fld[k];
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    wrelease(w);
    delete w;
    return wfail(LBM_ERR_CUDA, std::string("lbm_wing_create: ") + cudaGetErrorString(e));
  }
  *out = w;
  return LBM_OK;
}

lbm_status lbm_wing_destroy(lbm_wing *w) {
  if (!w) return LBM_OK;
  cudaSetDevice(w->cfg.device);
  cudaDeviceSynchronize();
  wrelease(w);
  delete w;
  return LBM_OK;
}

lbm_status lbm_wing_init(lbm_wing *w, const double state[4]) {
  if (!w || !state) return wfail(LBM_ERR_ARG, "null argument");
  WCUDA(cudaSetDevice(w->cfg.device));
  lbm_status st = build_mask(w, state);
  if (st != LBM_OK) return st;
  w->cur = 0;
  lbmw::wing_init_kernel<<<lbmk::cell_grid(w->n), 256>>>(w->f[0], w->mask, (int)w->n, (float)w->cfg.u0);
  WCUDA(cudaGetLastError());
  return LBM_OK;
}

lbm_status lbm_wing_step(lbm_wing *w, int32_t report, const double state[4], double load[3]) {
  lbmh::Range range_("lbm_wing_step");
  if (!w || !state || !load) return wfail(LBM_ERR_ARG, "null argument");
  WCUDA(cudaSetDevice(w->cfg.device));
  lbm_status st = build_mask(w, state);
  if (st != LBM_OK) return st;
  const lbm_wing_config &c = w->cfg;
  lbmw::WingArgs a{};
  a.fin = w->f[w->cur];
  a.fout = w->f[1 - w->cur];
  a.mask = w->mask;
  a.load = w->load;
  for (int k = 0; k < 5; ++k) a.fld[k] = w->fld[k];
  a.nx = c.nx;
  a.ny = c.ny;
  a.nz = c.nz;
  a.n = (int)w->n;
  a.x_ea = (float)c.x_ea;
  a.y_ea = (float)c.y_ea;
  a.h = (float)state[0];
  a.dh = (float)state[2];
  a.da = (float)state[3];
  a.u0 = (float)c.u0;
  a.sponge_start = (float)c.sponge_start;
  a.inv_sponge_len = (float)(1.0 / ((double)c.nx - c.sponge_start));
  a.sponge_strength = (float)c.sponge_strength;
  a.omega_bgk = (float)(1.0 / (3.0 * c.nu + 0.5));
  a.tau0 = (float)(3.0 * c.nu + 0.5);
  a.smag_c = (float)(25.456 * c.cs * c.cs);
  a.magic = (float)c.magic;
  WCUDA(cudaMemsetAsync(w->load, 0, 3 * sizeof(double)));
  switch (c.collision) {
    case LBM_BGK: launch_wing<lbmk::COLL_BGK>(w, a, report != 0); break;
    case LBM_TRT: launch_wing<lbmk::COLL_TRT>(w, a, report != 0); break;
    default: launch_wing<lbmk::COLL_LES>(w, a, report != 0); break;
  }
  WCUDA(cudaGetLastError());
  WCUDA(cudaMemcpy(load, w->load, 3 * sizeof(double), cudaMemcpyDeviceToHost));
  w->cur ^= 1;
  return LBM_OK;
}

lbm_status lbm_wing_set_physics(lbm_wing *w, int32_t collision, double nu) {
  if (!w) return wfail(LBM_ERR_ARG, "null argument");
  lbm_wing_config c = w->cfg;
  c.collision = collision;
  c.nu = nu;
  lbm_status st = wvalidate(c);
  if (st != LBM_OK) return st;
  w->cfg = c;
  return LBM_OK;
}

lbm_status lbm_wing_field(lbm_wing *w, int32_t id, float **ptr) {
  if (!w || !ptr) return wfail(LBM_ERR_ARG, "null argument");
  if (id < 0 || id >= 5) return wfail(LBM_ERR_ARG, "field id out of range (ux, uy, uz, p, vmag)");
  *ptr = w->fld[id];
  return LBM_OK;
}

lbm_status lbm_wing_populations(lbm_wing *w, float *host, int32_t set) {
  if (!w || !host) return wfail(LBM_ERR_ARG, "null argument");
  WCUDA(cudaSetDevice(w->cfg.device));
  const size_t fb = (size_t)19 * w->n * sizeof(float);
  if (set) WCUDA(cudaMemcpy(w->f[w->cur], host, fb, cudaMemcpyHostToDevice));
  else WCUDA(cudaMemcpy(host, w->f[w->cur], fb, cudaMemcpyDeviceToHost));
  return LBM_OK;
}

lbm_status lbm_wing_mask(lbm_wing *w, const double state[4], uint8_t *host) {
  if (!w || !state || !host) return wfail(LBM_ERR_ARG, "null argument");
  WCUDA(cudaSetDevice(w->cfg.device));
  lbm_status st = build_mask(w, state);
  if (st != LBM_OK) return st;
  WCUDA(cudaMemcpy(host, w->mask, (size_t)w->n, cudaMemcpyDeviceToHost));
  return LBM_OK;
}

lbm_status lbm_wing_set_output_stride(lbm_wing *w, int32_t stride) {
  if (!w) return wfail(LBM_ERR_ARG, "null argument");
  if (stride < 1) return wfail(LBM_ERR_ARG, "stride must be >= 1");
  WCUDA(cudaSetDevice(w->cfg.device));
  WCUDA(cudaDeviceSynchronize());
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
    WCUDA(cudaMallocManaged(&w->out[k], m * sizeof(float), cudaMemAttachGlobal));
    WCUDA(cudaMemset(w->out[k], 0, m * sizeof(float)));
  }
  return set_ptrs(w);
}

lbm_status lbm_wing_output(lbm_wing *w, int32_t id, float **ptr, int64_t *count) {
  if (!w || !ptr || !count) return wfail(LBM_ERR_ARG, "null argument");
  if (id < 0 || id >= 5) return wfail(LBM_ERR_ARG, "output id out of range (ux, uy, uz, p, vmag)");
  *ptr = w->out[id];
  *count = (int64_t)w->out_dims[0] * w->out_dims[1] * w->out_dims[2];
  return LBM_OK;
}

lbm_status lbm_wing_update_output(lbm_wing *w) {
  if (!w) return wfail(LBM_ERR_ARG, "null argument");
  if (w->stride <= 1) return LBM_OK;
  WCUDA(cudaSetDevice(w->cfg.device));
  const int m = w->out_dims[0] * w->out_dims[1] * w->out_dims[2];
  lbmw::wing_coarsen_kernel<<<lbmk::cell_grid(m), 256>>>(w->ptrs, w->ptrs + 5, w->cfg.nx, w->cfg.ny, w->stride,
                                                         w->out_dims[0], w->out_dims[1], m);
  WCUDA(cudaGetLastError());
  return LBM_OK;
}

}  // extern "C"
