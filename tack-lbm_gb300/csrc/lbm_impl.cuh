// lbm_impl.cuh - launch helpers, instantiated once per storage precision.
#pragma once

#include "lbm_device.cuh"
#include "lbm_host.h"

namespace lbmh {

using namespace lbmk;

template <typename S>
StepArgs<S> make_args(const Ctx &c) {
  using P = typename StepArgs<S>::P;
  const lbm_config &g = c.cfg;
  StepArgs<S> a{};
  S *F = static_cast<S *>(c.F);
  for (int q = 0; q < Q; ++q) a.slot[q] = F + (size_t)q * (size_t)c.n;
  a.nx = g.nx;
  a.ny = g.ny;
  a.nz = g.nz;
  a.nxy = g.nx * g.ny;
  a.geo = make_geo(g);
  a.lateral = g.lateral;
  a.vertical = g.vertical;
  a.u_lid = (P)g.u_lid;
  a.u0 = (P)g.u0;
  a.sponge_start = (P)g.sponge_start;
  a.sponge_strength = (P)g.sponge_strength;
  a.inv_sponge_len = (P)(1.0 / ((double)g.nx - g.sponge_start));
  a.omega_rot = (P)c.omega_rot;
  a.omega_bgk = (P)(1.0 / (3.0 * g.nu + 0.5));
  a.tau0 = (P)(3.0 * g.nu + 0.5);
  a.smag_c = (P)(25.456 * g.cs * g.cs);
  a.magic = (P)g.magic;
  for (int k = 0; k < LBM_NUM_FIELDS; ++k) a.fld[k] = c.fld[k];
  a.partials = c.partials;
  a.special = c.special;
  a.special_list = c.special_list;
  a.gx = c.gx;
  a.gy = c.gy;
  return a;
}

template <typename S, int COLL, bool REPORT, bool ODD>
cudaError_t launch_variant(const Ctx &c, const StepArgs<S> &a, cudaStream_t st) {
  const dim3 block(BX, BY);
  const dim3 grid(c.gx, c.gy, c.cfg.nz);
  cudaEvent_t *ev = c.ev && c.ev_used < c.ev_cap ? c.ev + 3 * c.ev_used : nullptr;
  if (ev) cudaEventRecord(ev[0], st);
  bulk_kernel<S, COLL, REPORT, ODD><<<grid, block, 0, st>>>(a);
  if (ev) cudaEventRecord(ev[1], st);
  if (c.nspecial > 0) generic_kernel<S, COLL, REPORT, ODD><<<c.nspecial, block, 0, st>>>(a);
  if (ev) cudaEventRecord(ev[2], st);
  return cudaGetLastError();
}

template <typename S, int COLL>
cudaError_t launch_coll(const Ctx &c, const StepArgs<S> &a, bool report, cudaStream_t st) {
  if (report) return c.odd_next ? launch_variant<S, COLL, true, true>(c, a, st)
                                : launch_variant<S, COLL, true, false>(c, a, st);
  return c.odd_next ? launch_variant<S, COLL, false, true>(c, a, st)
                    : launch_variant<S, COLL, false, false>(c, a, st);
}

template <typename S>
cudaError_t launch_step(const Ctx &c, bool report, cudaStream_t st) {
  const StepArgs<S> a = make_args<S>(c);
  cudaError_t e;
  switch (c.cfg.collision) {
    case LBM_BGK: e = launch_coll<S, COLL_BGK>(c, a, report, st); break;
    case LBM_TRT: e = launch_coll<S, COLL_TRT>(c, a, report, st); break;
    default: e = launch_coll<S, COLL_LES>(c, a, report, st); break;
  }
  if (e != cudaSuccess) return e;
  return report ? launch_finalize(c, st) : cudaSuccess;
}

template <typename S>
cudaError_t launch_init(const Ctx &c, double seed_amp, cudaStream_t st) {
  init_kernel<S><<<cell_grid(c.n), 256, 0, st>>>(make_args<S>(c), (float)seed_amp, (int)c.n);
  return cudaGetLastError();
}

template <typename S>
cudaError_t launch_init_random(const Ctx &c, double rho_sigma, double u_noise, uint64_t seed,
                               cudaStream_t st) {
  init_random_kernel<S><<<cell_grid(c.n), 256, 0, st>>>(make_args<S>(c), (float)rho_sigma,
                                                         (float)u_noise, splitmix64(seed), (int)c.n);
  return cudaGetLastError();
}

template <typename S>
cudaError_t launch_import(const Ctx &c, const void *src, int dtype, cudaStream_t st) {
  if (dtype == LBM_F64)
    import_kernel<S, double><<<cell_grid(c.n), 256, 0, st>>>(make_args<S>(c), (const double *)src, (int)c.n);
  else
    import_kernel<S, float><<<cell_grid(c.n), 256, 0, st>>>(make_args<S>(c), (const float *)src, (int)c.n);
  return cudaGetLastError();
}

template <typename S>
cudaError_t launch_export(const Ctx &c, void *dst, int dtype, cudaStream_t st) {
  if (dtype == LBM_F64)
    export_kernel<S, double><<<cell_grid(c.n), 256, 0, st>>>(make_args<S>(c), (double *)dst, (int)c.n,
                                                              c.odd_next);
  else
    export_kernel<S, float><<<cell_grid(c.n), 256, 0, st>>>(make_args<S>(c), (float *)dst, (int)c.n,
                                                             c.odd_next);
  return cudaGetLastError();
}

#define LBM_INSTANTIATE(S)                                                                    \
  template cudaError_t launch_step<S>(const Ctx &, bool, cudaStream_t);                       \
  template cudaError_t launch_init<S>(const Ctx &, double, cudaStream_t);                     \
  template cudaError_t launch_init_random<S>(const Ctx &, double, double, uint64_t, cudaStream_t); \
  template cudaError_t launch_import<S>(const Ctx &, const void *, int, cudaStream_t);        \
  template cudaError_t launch_export<S>(const Ctx &, void *, int, cudaStream_t);

}  // namespace lbmh
