// lbm_impl.cuh - launch helpers, instantiated once per storage precision.
#pragma once

#include "lbm_device.cuh"
#include "lbm_host.h"
#include "lbm_stream.cuh"

#include <algorithm>

namespace lbmh {

using namespace lbmk;

template <typename S>
StepArgs<S> make_args(const Ctx &c) {
  using P = typename StepArgs<S>::P;
  const lbm_config &g = c.cfg;
  StepArgs<S> a{};
  S *F = static_cast<S *>(c.F);
  for (int q = 0; q < Q; ++q) a.slot[q] = F + (size_t)q * (size_t)c.n;
  a.F = F;
  a.n = (uint32_t)c.n;
  a.blk = c.blocked;
  a.rowp = c.rowp;
  {
    const uint32_t planep = c.rowp * (uint32_t)g.ny;
    a.bstep[0] = (int)(0u - c.rowp);
    a.bstep[1] = (int)c.rowp;
    a.bstep[2] = (int)(0u - planep);
    a.bstep[3] = (int)planep;
    a.bwrap[0] = (int)((uint32_t)(g.ny - 1) * c.rowp);
    a.bwrap[1] = (int)(0u - (uint32_t)(g.ny - 1) * c.rowp);
    a.bwrap[2] = (int)((uint32_t)(g.nz - 1) * planep);
    a.bwrap[3] = (int)(0u - (uint32_t)(g.nz - 1) * planep);
  }
  // a storage type with the block layout has no flat slot-layout form
  a.flat = blocked_layout(sizeof(S)) ? c.blocked
                                     : 19 * c.n <= (int64_t)UINT32_MAX && !(g.flags & LBM_FLAG_SLOT_POINTERS);
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
  a.wall_ox = (P)g.ox;
  a.wall_oy = (P)g.oy;
  a.wall_inv_r = g.r != 0.0 ? (P)(1.0 / g.r) : (P)0;
  a.omega_bgk = (P)(1.0 / (3.0 * g.nu + 0.5));
  a.tau0 = (P)(3.0 * g.nu + 0.5);
  a.smag_c = (P)(25.456 * g.cs * g.cs);
  a.magic = (P)g.magic;
  for (int k = 0; k < LBM_NUM_FIELDS; ++k) a.fld[k] = c.fld[k];
  a.aux = c.cfg.heat ? c.aux : nullptr;
  a.partials = c.partials;
  for (int k = 0; k < 3; ++k) {
    a.reach_lo[k] = c.reach_lo[k];
    a.reach_hi[k] = c.reach_hi[k];
  }
  a.reach_any = c.reach_any;
  a.masks = c.wmasks;
  a.gx = c.gx;
  a.gy = c.gy;
  return a;
}

// Persistent grid of the bulk-copy kernel: every SM filled to its occupancy.
template <typename S, int COLL, bool REPORT, bool ODD>
int stream_grid(const Ctx &c) {
  constexpr int MAXDEV = 64;
  static int per_sm[MAXDEV] = {};
  const int dev = c.cfg.device < MAXDEV ? c.cfg.device : 0;
  if (per_sm[dev] == 0) {
    auto kern = stream_kernel<S, COLL, REPORT, ODD>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Layout<S>::BYTES);
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, SW + 32, Layout<S>::BYTES);
    per_sm[dev] = nb > 0 ? nb : 1;
  }
  const long long g = (long long)per_sm[dev] * c.num_sms;
  return (int)(g < c.nseg ? g : c.nseg);
}

template <typename S, int COLL, bool REPORT, bool ODD>
cudaError_t launch_variant(const Ctx &c, const StepArgs<S> &a, cudaStream_t st, int64_t *rows) {
  cudaEvent_t *ev = c.ev && c.ev_used < c.ev_cap ? c.ev + 3 * c.ev_used : nullptr;
  if (ev) cudaEventRecord(ev[0], st);
  if (c.use_stream) {
    StreamArgs<S> sa;
    sa.a = a;
    sa.nseg_x = c.nseg_x;
    sa.nseg = c.nseg;
    sa.seg_mask = c.seg_mask;
    sa.masks = c.masks;
    sa.error = c.error;
    sa.wait_limit = c.wait_limit;
    sa.starve = c.starve_next;
    const int grid = stream_grid<S, COLL, REPORT, ODD>(c);
    stream_kernel<S, COLL, REPORT, ODD><<<grid, SW + 32, Layout<S>::BYTES, st>>>(sa);
    *rows = grid;
    if (ev) cudaEventRecord(ev[1], st);
  } else {
    const dim3 block(BX, BY);
    const dim3 grid(c.gx, c.gy, c.cfg.nz);
    const int64_t fblocks = (int64_t)grid.x * grid.y * grid.z;
    const int gblocks = (c.nspecial + BY - 1) / BY;
    if (gblocks > 0) {
      // the special warps run beside the fast kernel: their cells' memory is disjoint
      cudaEventRecord(c.fork, st);
      cudaStreamWaitEvent(c.side, c.fork, 0);
      general_kernel<S, COLL, REPORT, ODD><<<gblocks, block, 0, c.side>>>(a, c.special, c.nspecial, c.wx,
                                                                         (int)fblocks);
      cudaEventRecord(c.join, c.side);
    }
    {
      constexpr int TX = tile_warps_x<S>(), TY = BY / TX;
      const dim3 tiles((c.cfg.nx + BX * TX - 1) / (BX * TX), (c.cfg.ny + TY - 1) / TY, c.cfg.nz);
      step_kernel<S, COLL, REPORT, ODD><<<tiles, block, 0, st>>>(a);
    }
    if (ev) cudaEventRecord(ev[1], st);
    if (gblocks > 0) cudaStreamWaitEvent(st, c.join, 0);
    *rows = 0;
    if (REPORT) {
      // the monitor sums, read back from the fields just written
      const int sblocks = (int)std::min<int64_t>((c.n + SUM_THREADS * 16 - 1) / (SUM_THREADS * 16),
                                                 (int64_t)c.num_sms * SUM_BLOCKS_PER_SM);
      SumBox box{};
      for (int k = 0; k < 3; ++k) {
        box.lo[k] = c.reach_lo[k];
        box.hi[k] = c.reach_hi[k];
      }
      box.any = c.reach_any;
      box.nx = c.cfg.nx;
      box.ny = c.cfg.ny;
      field_sums_kernel<<<sblocks, SUM_THREADS, 0, st>>>(c.fld_dev, (int)c.n, box, c.partials, c.ticket, c.sums);
      *rows = 0;  // finalized by the kernel's last block
    }
    (void)fblocks;
  }
  if (ev) cudaEventRecord(ev[2], st);
  return cudaGetLastError();
}

template <typename S, int COLL>
cudaError_t launch_coll(const Ctx &c, const StepArgs<S> &a, bool report, cudaStream_t st, int64_t *rows) {
  if (report) return c.odd_next ? launch_variant<S, COLL, true, true>(c, a, st, rows)
                                : launch_variant<S, COLL, true, false>(c, a, st, rows);
  return c.odd_next ? launch_variant<S, COLL, false, true>(c, a, st, rows)
                    : launch_variant<S, COLL, false, false>(c, a, st, rows);
}

template <typename S>
cudaError_t launch_step(const Ctx &c, bool report, cudaStream_t st) {
  const StepArgs<S> a = make_args<S>(c);
  cudaError_t e;
  int64_t rows = 0;
  switch (c.cfg.collision) {
    case LBM_BGK: e = launch_coll<S, COLL_BGK>(c, a, report, st, &rows); break;
    case LBM_TRT: e = launch_coll<S, COLL_TRT>(c, a, report, st, &rows); break;
    default: e = launch_coll<S, COLL_LES>(c, a, report, st, &rows); break;
  }
  if (e != cudaSuccess) return e;
  return report && rows > 0 ? launch_finalize(c, rows, st) : cudaSuccess;
}

template <typename S>
cudaError_t launch_warp_masks(const Ctx &c, cudaStream_t st) {
  if (!c.reach_any) return cudaSuccess;
  warp_mask_kernel<S><<<dim3(c.gx, c.cfg.ny, c.cfg.nz), BX, 0, st>>>(make_args<S>(c), c.wmasks);
  return cudaGetLastError();
}

template <typename S>
cudaError_t launch_link_masks(const Ctx &c, cudaStream_t st) {
  if (c.nmasked == 0) return cudaSuccess;
  link_mask_kernel<S><<<c.nmasked, SW, 0, st>>>(make_args<S>(c), c.nseg_x, c.seg_list, c.nmasked, c.masks);
  return cudaGetLastError();
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
  template cudaError_t launch_export<S>(const Ctx &, void *, int, cudaStream_t);                \
  template cudaError_t launch_link_masks<S>(const Ctx &, cudaStream_t);                       \
  template cudaError_t launch_warp_masks<S>(const Ctx &, cudaStream_t);

}  // namespace lbmh
