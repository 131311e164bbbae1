// lbm_host.h - host-side state shared by the C ABI and the per-precision kernel units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/lbm_gb300.h"

#if defined(__has_include)
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define LBM_HAVE_NVTX 1
#endif
#endif

namespace lbmh {

// An NVTX range over one C-ABI call, named after the entry point, so that
// timeline and kernel profilers can group a step's launches (ncu --nvtx
// --nvtx-include "lbm_step/"). NVTX is header-only and does nothing unless a
// tool is attached; without the header the range is empty.
struct Range {
  explicit Range(const char *name) {
#ifdef LBM_HAVE_NVTX
    nvtxRangePushA(name);
#else
    (void)name;
#endif
  }
  ~Range() {
#ifdef LBM_HAVE_NVTX
    nvtxRangePop();
#endif
  }
  Range(const Range &) = delete;
  Range &operator=(const Range &) = delete;
};

// Everything the launch helpers need about one solver.
struct Ctx {
  lbm_config cfg;
  int64_t n;                 // cells
  void *F;                   // the populations, storage precision cfg.storage
  int blocked;               // F in the block layout (19 x npos), else the slot layout (19 x n)
  int64_t npos;              // block layout: cells with each row padded to whole 32-cell blocks
  uint32_t rowp;             // block layout: elements per lattice row
  float *fld[LBM_NUM_FIELDS];
  float **fld_dev;           // the field pointers in device memory (for the sums kernel)
  float2 *partials;          // 8 compensated float pairs per block (report steps)
  double *stage;             // finalize stage: 8 doubles per finalize block
  double *sums;              // 8 doubles: the last report step's FP64 sums
  int reach_lo[3], reach_hi[3], reach_any;  // cells that may be solid or next to solid
  uint32_t *wmasks;          // link masks of the 32-cell warps within the obstacle's reach
  int *special;              // row-segment ids of the warps the general kernel updates (lid rows)
  int nspecial;              // how many
  int64_t special_cells;     // cells in them
  int wx;                    // 32-cell row segments per row
  cudaStream_t side;         // high-priority stream the general kernel overlaps on
  cudaEvent_t fork, join;
  int gx, gy;                // blocks along x and y (32 x 4 cells each)
  int64_t nblocks;           // gx*gy*nz
  int odd_next;              // 1: the next step reads neighbours (state in "even view")
  double omega_rot;
  int out_stride;            // output grid subsampling (1: aliases fld)
  int out_dims[3];
  int nout;                  // output fields: 5, or 6 with temperature
  float *out[LBM_MAX_OUTPUTS];  // coarse ux, uy, uz, p, vmag, temp (owned when out_stride > 1)
  // D3Q7 temperature (cfg.heat): A/B populations, the flow's per-cell moments, fields
  float *g[2];
  int g_cur;                 // g[g_cur] holds the current temperature populations
  float4 *aux;               // (ux, uy, uz, tau) per fluid cell, written by the flow step
  float *heat_fld[LBM_NUM_HEAT_FIELDS];
  // lbm_run: two quiet steps (odd + even, with their lid-row and heat launches)
  // captured as one CUDA graph per starting parity, replayed while the
  // arguments the kernels took stay the same
  cudaStream_t capture;
  cudaGraphExec_t pair_graph[2];
  // optional kernel timing: events around the bulk and generic launches
  cudaEvent_t *ev;           // 3 events per step in a ring (bulk start, bulk end/generic start, generic end)
  int ev_cap, ev_used;
  int64_t bulk_cells, generic_cells;
  // bulk-copy (TMA) path: row segments of lbmk::SW cells
  int use_stream;            // 1 when nx suits 16-byte row pieces
  long long wait_limit;      // bulk-copy kernel: mbarrier polls before a wait gives up
  int starve_next;           // test hook: the next bulk-copy step issues no copies (lbm_test_bulkcopy_stall)
  int nseg_x, nseg;          // segments per row, segments in the lattice
  int *seg_mask;             // per segment: first link-mask word or -1
  int *seg_list;             // the masked segments
  uint32_t *masks;           // SW words per masked segment
  int nmasked;
  unsigned int *error;       // set by a kernel whose copy wait gave up
  unsigned int *ticket;      // blocks of field_sums_kernel done (the last one finalizes and resets it)
  int num_sms;
  int64_t partial_rows;      // capacity of `partials` in rows of 8 doubles
};

constexpr int FINALIZE_BLOCKS = 128;

// per-precision entry points (explicitly instantiated in lbm_kernels_<p>.cu)
template <typename S> cudaError_t launch_step(const Ctx &c, bool report, cudaStream_t st);
template <typename S> cudaError_t launch_init(const Ctx &c, double seed_amp, cudaStream_t st);
template <typename S> cudaError_t launch_init_random(const Ctx &c, double rho_sigma, double u_noise,
                                                     uint64_t seed, cudaStream_t st);
// src/dst: device pointers to 19*n values of float (dtype LBM_F32) or double (LBM_F64)
template <typename S> cudaError_t launch_import(const Ctx &c, const void *src, int dtype, cudaStream_t st);
template <typename S> cudaError_t launch_export(const Ctx &c, void *dst, int dtype, cudaStream_t st);
template <typename S> cudaError_t launch_link_masks(const Ctx &c, cudaStream_t st);
template <typename S> cudaError_t launch_warp_masks(const Ctx &c, cudaStream_t st);

cudaError_t launch_finalize(const Ctx &c, int64_t rows, cudaStream_t st);
cudaError_t launch_mask(const Ctx &c, uint8_t *dst_dev, cudaStream_t st);
cudaError_t launch_coarsen(const Ctx &c, cudaStream_t st);
cudaError_t launch_heat(const Ctx &c, bool report, cudaStream_t st);
cudaError_t launch_jacobian(const Ctx &c, float *jac, float inv_h, cudaStream_t st);
cudaError_t launch_vortq(const Ctx &c, const float *jac, float *vort, float *q, int at_cells, cudaStream_t st);
cudaError_t launch_vortq_direct(const Ctx &c, float inv_h, float *vort, float *q, int at_cells, cudaStream_t st);
// the full-resolution field output k shows (fld[k], or the temperature)
inline float *output_source(const Ctx &c, int k) { return k < 5 ? c.fld[k] : c.heat_fld[LBM_TEMP]; }

// message returned by lbm_last_error() on this thread
void set_last_error(const std::string &msg);

}  // namespace lbmh
