// lbm_api.cu - the C ABI (include/lbm_gb300.h): solver handles, buffers, dispatch.
//
// One solver owns: the in-place AA population buffer (device memory), the 13
// diagnostic fields (CUDA managed memory, as the reference's ManagedArray,
// lbm.py:525-541), the per-block FP64 partial sums of report steps and the
// block classification (bulk vs generic) of its geometry.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "lbm_device.cuh"
#include "lbm_host.h"
#include "lbm_stream.cuh"

using lbmh::Ctx;

struct lbm_solver {
  Ctx c;
  int64_t bytes = 0;
  int64_t steps = 0;
  bool reported = false;
};

namespace {

thread_local std::string g_err;

lbm_status fail(lbm_status s, const std::string &msg) {
  g_err = msg;
  return s;
}

#define LBM_CUDA(call)                                                                         \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess)                                                                     \
      return fail(LBM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));           \
  } while (0)

size_t storage_bytes(int storage) {
  switch (storage) {
    case LBM_F16: return sizeof(__half);
    case LBM_BF16: return sizeof(__nv_bfloat16);
    case LBM_F64: return sizeof(double);
    default: return sizeof(float);
  }
}

lbm_status validate(const lbm_config &g) {
  if (g.nx < 1 || g.ny < 1 || g.nz < 1) return fail(LBM_ERR_ARG, "lattice sizes must be >= 1");
  const int64_t n = (int64_t)g.nx * g.ny * g.nz;
  if (n > 2147483647LL) return fail(LBM_ERR_ARG, "more than 2^31-1 cells");
  if ((g.ny + lbmk::BY - 1) / lbmk::BY > 65535 || g.nz > 65535)
    return fail(LBM_ERR_ARG, "ny/4 and nz must be <= 65535");
  if (g.collision < LBM_BGK || g.collision > LBM_LES)
    return fail(LBM_ERR_ARG, "unknown collision model (bgk=0, trt=1, les=2)");
  if (g.obstacle < LBM_NO_OBSTACLE || g.obstacle > LBM_HEATSINK)
    return fail(LBM_ERR_ARG, "unknown obstacle (none=0, cylinder=1, sphere=2, box=3, heatsink=4)");
  for (double v : g.sink)
    if (!std::isfinite(v) || v < 0.0 || v > 1e9) return fail(LBM_ERR_ARG, "heat sink sizes must be finite and >= 0");
  if (g.obstacle == LBM_HEATSINK && !(g.sink[7] >= 1.0)) return fail(LBM_ERR_ARG, "heat sink fin pitch must be >= 1");
  if (g.heat) {
    if (g.storage != LBM_F32) return fail(LBM_ERR_ARG, "heat needs FP32 population storage");
    if (!(std::isfinite(g.alpha) && g.alpha >= 0.0 && std::isfinite(g.heat_nu)))
      return fail(LBM_ERR_ARG, "heat diffusivity must be finite and >= 0");
  }
  if (g.lateral < LBM_PERIODIC || g.lateral > LBM_LID)
    return fail(LBM_ERR_ARG, "unknown lateral policy (periodic=0, slip=1, lid=2)");
  if (g.vertical != LBM_PERIODIC && g.vertical != LBM_SLIP)
    return fail(LBM_ERR_ARG, "unknown vertical policy (periodic=0, slip=1)");
  if (g.storage < LBM_F32 || g.storage > LBM_F64)
    return fail(LBM_ERR_ARG, "unknown storage (f32=0, f16=1, bf16=2, f64=3)");
  if (!(std::isfinite(g.nu) && g.nu > 0.0)) return fail(LBM_ERR_ARG, "nu must be finite and > 0");
  if (!(std::isfinite(g.cs) && g.cs >= 0.0)) return fail(LBM_ERR_ARG, "cs must be finite and >= 0");
  const double vals[] = {g.magic, g.ox, g.oy, g.oz, g.r, g.hx, g.hy, g.hz, g.u0,
                         g.sponge_start, g.sponge_strength, g.u_lid, g.omega_rot};
  for (double v : vals)
    if (!std::isfinite(v)) return fail(LBM_ERR_ARG, "configuration values must be finite");
  return LBM_OK;
}

// Cells that may be solid or have a solid neighbour lie in [lo, hi] along each axis.
struct Range {
  int64_t lo, hi;
};

void obstacle_box(const lbm_config &g, Range r[3], bool &any) {
  double c[3] = {g.ox, g.oy, g.oz}, h[3] = {0, 0, 0};
  any = true;
  if (g.obstacle == LBM_CYLINDER || g.obstacle == LBM_SPHERE) {
    h[0] = h[1] = h[2] = g.r;
    if (!(g.r > 0)) any = false;
  } else if (g.obstacle == LBM_BOX) {
    h[0] = g.hx;
    h[1] = g.hy;
    h[2] = g.hz;
    if (!(g.hx > 0 && g.hy > 0 && g.hz > 0)) any = false;
  } else if (g.obstacle == LBM_HEATSINK) {
    // duct walls at y = 0 and ny - 1 along the whole lattice
    const int64_t dims[3] = {g.nx, g.ny, g.nz};
    for (int k = 0; k < 3; ++k) r[k] = {0, dims[k] - 1};
    return;
  } else {
    any = false;
  }
  const int64_t dims[3] = {g.nx, g.ny, g.nz};
  for (int k = 0; k < 3; ++k) {
    if (k == 2 && g.obstacle == LBM_CYLINDER) {
      r[k] = {0, dims[k] - 1};
      continue;
    }
    const double lo = std::floor(c[k] - h[k]) - 2.0, hi = std::ceil(c[k] + h[k]) + 2.0;
    r[k].lo = (int64_t)std::max(lo, -1e15);
    r[k].hi = (int64_t)std::min(hi, 1e15);
    const bool periodic = k == 0 || (k == 1 && g.lateral == LBM_PERIODIC) ||
                          (k == 2 && g.vertical == LBM_PERIODIC);
    // a neighbour across a periodic boundary: widen to the whole axis
    if (periodic && (r[k].lo <= 0 || r[k].hi >= dims[k] - 1)) r[k] = {0, dims[k] - 1};
    if (r[k].hi < 0 || r[k].lo > dims[k] - 1) any = false;
  }
}

// The obstacle's reach box (clamped to the lattice), the link masks of the
// 32-cell warps inside it, and the lid rows the general kernel updates.
lbm_status set_reach(Ctx &c) {
  Range box[3];
  bool any;
  obstacle_box(c.cfg, box, any);
  const lbm_config &g = c.cfg;
  const int64_t dims[3] = {g.nx, g.ny, g.nz};
  for (int k = 0; k < 3; ++k) {
    c.reach_lo[k] = (int)std::max<int64_t>(box[k].lo, 0);
    c.reach_hi[k] = (int)std::min<int64_t>(box[k].hi, dims[k] - 1);
    if (c.reach_lo[k] > c.reach_hi[k]) any = false;
  }
  c.reach_any = any ? 1 : 0;
  cudaFree(c.wmasks);
  c.wmasks = nullptr;
  if (c.reach_any) {
    const int64_t nw = c.reach_hi[0] / lbmk::BX - c.reach_lo[0] / lbmk::BX + 1;
    const int64_t words = nw * (c.reach_hi[1] - c.reach_lo[1] + 1) * (c.reach_hi[2] - c.reach_lo[2] + 1) *
                          lbmk::BX;
    LBM_CUDA(cudaMalloc(&c.wmasks, (size_t)words * sizeof(uint32_t)));
    LBM_CUDA(lbmh::launch_warp_masks<float>(c, 0));
    LBM_CUDA(cudaDeviceSynchronize());
  }
  c.wx = (g.nx + lbmk::BX - 1) / lbmk::BX;
  c.special_cells = 0;
  std::vector<int> list;
  if (g.lateral == LBM_LID)
    for (int z = 0; z < g.nz; ++z)
      for (int w = 0; w < c.wx; ++w) {
        list.push_back((z * g.ny + (g.ny - 1)) * c.wx + w);
        c.special_cells += std::min(lbmk::BX, g.nx - w * lbmk::BX);
      }
  cudaFree(c.special);
  c.special = nullptr;
  c.nspecial = (int)list.size();
  LBM_CUDA(cudaMalloc(&c.special, std::max<size_t>(1, list.size()) * sizeof(int)));
  if (!list.empty())
    LBM_CUDA(cudaMemcpy(c.special, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice));
  return LBM_OK;
}

// Row segments of the bulk-copy kernel within reach of the obstacle get link masks.
lbm_status classify_segments(lbm_solver *s) {
  Ctx &c = s->c;
  const lbm_config &g = c.cfg;
  cudaFree(c.seg_mask);
  cudaFree(c.seg_list);
  cudaFree(c.masks);
  c.seg_mask = nullptr;
  c.seg_list = nullptr;
  c.masks = nullptr;
  c.nmasked = 0;
  if (!c.use_stream) return LBM_OK;
  Range box[3];
  bool any;
  obstacle_box(g, box, any);
  std::vector<int> slot((size_t)c.nseg, -1), list;
  for (int z = 0; z < g.nz; ++z)
    for (int y = 0; y < g.ny; ++y)
      for (int sx = 0; sx < c.nseg_x; ++sx) {
        const int64_t x0 = (int64_t)sx * lbmk::SW;
        const int64_t x1 = std::min<int64_t>(x0 + lbmk::SW, g.nx) - 1;
        if (any && x1 >= box[0].lo && x0 <= box[0].hi && y >= box[1].lo && y <= box[1].hi &&
            z >= box[2].lo && z <= box[2].hi) {
          const int seg = (z * g.ny + y) * c.nseg_x + sx;
          slot[(size_t)seg] = (int)list.size() * lbmk::SW;
          list.push_back(seg);
        }
      }
  c.nmasked = (int)list.size();
  LBM_CUDA(cudaMalloc(&c.seg_mask, slot.size() * sizeof(int)));
  LBM_CUDA(cudaMemcpy(c.seg_mask, slot.data(), slot.size() * sizeof(int), cudaMemcpyHostToDevice));
  LBM_CUDA(cudaMalloc(&c.seg_list, std::max<size_t>(1, list.size()) * sizeof(int)));
  LBM_CUDA(cudaMalloc(&c.masks, std::max<size_t>(1, list.size()) * lbmk::SW * sizeof(uint32_t)));
  if (!list.empty()) {
    LBM_CUDA(cudaMemcpy(c.seg_list, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice));
    LBM_CUDA(lbmh::launch_link_masks<float>(c, 0));
    LBM_CUDA(cudaDeviceSynchronize());
  }
  return LBM_OK;
}

cudaError_t dispatch_step(const Ctx &c, bool report, cudaStream_t st) {
  switch (c.cfg.storage) {
    case LBM_F16: return lbmh::launch_step<__half>(c, report, st);
    case LBM_BF16: return lbmh::launch_step<__nv_bfloat16>(c, report, st);
    case LBM_F64: return lbmh::launch_step<double>(c, report, st);
    default: return lbmh::launch_step<float>(c, report, st);
  }
}

cudaError_t dispatch_init(const Ctx &c, double seed_amp, cudaStream_t st) {
  switch (c.cfg.storage) {
    case LBM_F16: return lbmh::launch_init<__half>(c, seed_amp, st);
    case LBM_BF16: return lbmh::launch_init<__nv_bfloat16>(c, seed_amp, st);
    case LBM_F64: return lbmh::launch_init<double>(c, seed_amp, st);
    default: return lbmh::launch_init<float>(c, seed_amp, st);
  }
}

cudaError_t dispatch_init_random(const Ctx &c, double rs, double un, uint64_t seed, cudaStream_t st) {
  switch (c.cfg.storage) {
    case LBM_F16: return lbmh::launch_init_random<__half>(c, rs, un, seed, st);
    case LBM_BF16: return lbmh::launch_init_random<__nv_bfloat16>(c, rs, un, seed, st);
    case LBM_F64: return lbmh::launch_init_random<double>(c, rs, un, seed, st);
    default: return lbmh::launch_init_random<float>(c, rs, un, seed, st);
  }
}

cudaError_t dispatch_import(const Ctx &c, const void *src, int dtype, cudaStream_t st) {
  switch (c.cfg.storage) {
    case LBM_F16: return lbmh::launch_import<__half>(c, src, dtype, st);
    case LBM_BF16: return lbmh::launch_import<__nv_bfloat16>(c, src, dtype, st);
    case LBM_F64: return lbmh::launch_import<double>(c, src, dtype, st);
    default: return lbmh::launch_import<float>(c, src, dtype, st);
  }
}

cudaError_t dispatch_export(const Ctx &c, void *dst, int dtype, cudaStream_t st) {
  switch (c.cfg.storage) {
    case LBM_F16: return lbmh::launch_export<__half>(c, dst, dtype, st);
    case LBM_BF16: return lbmh::launch_export<__nv_bfloat16>(c, dst, dtype, st);
    case LBM_F64: return lbmh::launch_export<double>(c, dst, dtype, st);
    default: return lbmh::launch_export<float>(c, dst, dtype, st);
  }
}

// Managed fields live in the GPU's HBM (the kernels write them every report
// step) and are read by the host in place: on a coherent Grace system the CPU
// reaches them over NVLink-C2C without migrating pages back. Advice failures
// (systems without these attributes) leave the default placement.
void place_on_device(void *p, size_t bytes, int device) {
  cudaMemLocation gpu{};
  gpu.type = cudaMemLocationTypeDevice;
  gpu.id = device;
  cudaMemLocation cpu{};
  cpu.type = cudaMemLocationTypeHost;
  cpu.id = 0;
  if (cudaMemAdvise(p, bytes, cudaMemAdviseSetPreferredLocation, gpu) != cudaSuccess) cudaGetLastError();
  if (cudaMemAdvise(p, bytes, cudaMemAdviseSetAccessedBy, cpu) != cudaSuccess) cudaGetLastError();
  if (cudaMemPrefetchAsync(p, bytes, gpu, 0, 0) != cudaSuccess) cudaGetLastError();
}

void release_output(Ctx &c) {
  if (c.out_stride > 1)
    for (int k = 0; k < c.nout; ++k) cudaFree(c.out[k]);
  for (int k = 0; k < LBM_MAX_OUTPUTS; ++k) c.out[k] = k < c.nout ? lbmh::output_source(c, k) : nullptr;
  c.out_stride = 1;
  c.out_dims[0] = c.cfg.nx;
  c.out_dims[1] = c.cfg.ny;
  c.out_dims[2] = c.cfg.nz;
}

// Forget the captured step graphs (after anything their kernels took as an
// argument has changed).
void drop_graphs(Ctx &c) {
  for (cudaGraphExec_t &g : c.pair_graph) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
}

void release_timing(Ctx &c) {
  if (c.ev) {
    for (int k = 0; k < 3 * c.ev_cap; ++k) cudaEventDestroy(c.ev[k]);
    delete[] c.ev;
  }
  c.ev = nullptr;
  c.ev_cap = c.ev_used = 0;
}

void release(lbm_solver *s) {
  Ctx &c = s->c;
  release_timing(c);
  release_output(c);
  cudaFree(c.seg_mask);
  cudaFree(c.seg_list);
  cudaFree(c.masks);
  cudaFree(c.error);
  cudaFree(c.ticket);
  cudaFree(c.special);
  cudaFree(c.wmasks);
  cudaFree(c.fld_dev);
  drop_graphs(c);
  if (c.capture) cudaStreamDestroy(c.capture);
  if (c.side) cudaStreamDestroy(c.side);
  if (c.fork) cudaEventDestroy(c.fork);
  if (c.join) cudaEventDestroy(c.join);
  cudaFree(c.F);
  for (int k = 0; k < LBM_NUM_FIELDS; ++k) cudaFree(c.fld[k]);
  cudaFree(c.g[0]);
  cudaFree(c.g[1]);
  cudaFree(c.aux);
  for (int k = 0; k < LBM_NUM_HEAT_FIELDS; ++k) cudaFree(c.heat_fld[k]);
  cudaFree(c.partials);
  cudaFree(c.stage);
  cudaFree(c.sums);
}

}  // namespace

// ---------------------------------------------------------------------------
// FP64 reduction of the per-block partial sums, in a fixed order (deterministic).

namespace lbmh {

void set_last_error(const std::string &msg) { g_err = msg; }

__global__ void finalize_stage(const float2 *partials, int64_t nb, double *stage) {
  __shared__ double sm[256][lbmk::NSUM];
  const int64_t chunk = (nb + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = (int64_t)blockIdx.x * chunk;
  const int64_t b1 = b0 + chunk < nb ? b0 + chunk : nb;
  double acc[lbmk::NSUM] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int64_t b = b0 + threadIdx.x; b < b1; b += blockDim.x)
    for (int k = 0; k < lbmk::NSUM; ++k) {
      const float2 p = partials[b * lbmk::NSUM + k];
      acc[k] += (double)p.x + (double)p.y;
    }
  for (int k = 0; k < lbmk::NSUM; ++k) sm[threadIdx.x][k] = acc[k];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int k = 0; k < lbmk::NSUM; ++k) sm[threadIdx.x][k] += sm[threadIdx.x + w][k];
    __syncthreads();
  }
  if (threadIdx.x < lbmk::NSUM) stage[blockIdx.x * lbmk::NSUM + threadIdx.x] = sm[0][threadIdx.x];
}

__global__ void finalize_last(const double *stage, int g, double *sums) {
  if (threadIdx.x < lbmk::NSUM) {
    double s = 0.0;
    for (int i = 0; i < g; ++i) s += stage[i * lbmk::NSUM + threadIdx.x];
    sums[threadIdx.x] = s;
  }
}

cudaError_t launch_finalize(const Ctx &c, int64_t rows, cudaStream_t st) {
  finalize_stage<<<FINALIZE_BLOCKS, 256, 0, st>>>(c.partials, rows, c.stage);
  finalize_last<<<1, 32, 0, st>>>(c.stage, FINALIZE_BLOCKS, c.sums);
  return cudaGetLastError();
}

__global__ void mask_kernel(lbmk::Geo geo, int nx, int ny, int n, uint8_t *out) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    int x, y, z;
    lbmk::decode(idx, nx, ny, x, y, z);
    out[idx] = lbmk::solid(geo, x, y, z) ? 1 : 0;
  }
}

// coarsen (lbm.py:516-522): dst[(k*my + j)*mx + i] = src[((k*s)*ny + j*s)*nx + i*s] per output field
struct CoarsenArgs {
  const float *src[LBM_MAX_OUTPUTS];
  float *dst[LBM_MAX_OUTPUTS];
  int count;
};

__global__ void coarsen_kernel(CoarsenArgs a, int nx, int ny, int s, int mx, int my, int m) {
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < m; idx += gridDim.x * blockDim.x) {
    const int i = idx % mx, j = (idx / mx) % my, k = idx / (mx * my);
    const int src = ((k * s) * ny + j * s) * nx + i * s;
#pragma unroll
    for (int f = 0; f < LBM_MAX_OUTPUTS; ++f)
      if (f < a.count) a.dst[f][idx] = a.src[f][src];
  }
}

cudaError_t launch_coarsen(const Ctx &c, cudaStream_t st) {
  if (c.out_stride <= 1) return cudaSuccess;
  CoarsenArgs a{};
  a.count = c.nout;
  for (int f = 0; f < c.nout; ++f) {
    a.src[f] = output_source(c, f);
    a.dst[f] = c.out[f];
  }
  const int m = c.out_dims[0] * c.out_dims[1] * c.out_dims[2];
  coarsen_kernel<<<lbmk::cell_grid(m), 256, 0, st>>>(a, c.cfg.nx, c.cfg.ny, c.out_stride, c.out_dims[0],
                                                     c.out_dims[1], m);
  return cudaGetLastError();
}

cudaError_t launch_mask(const Ctx &c, uint8_t *dst, cudaStream_t st) {
  mask_kernel<<<lbmk::cell_grid(c.n), 256, 0, st>>>(lbmk::make_geo(c.cfg), c.cfg.nx, c.cfg.ny, (int)c.n, dst);
  return cudaGetLastError();
}

}  // namespace lbmh

// ---------------------------------------------------------------------------
// C ABI

extern "C" {

int32_t lbm_abi_version(void) { return 2; }

const char *lbm_last_error(void) { return g_err.c_str(); }

lbm_status lbm_create(const lbm_config *cfg, lbm_solver **out) {
  if (!cfg || !out) return fail(LBM_ERR_ARG, "null argument");
  *out = nullptr;
  lbm_status st = validate(*cfg);
  if (st != LBM_OK) return st;
  LBM_CUDA(cudaSetDevice(cfg->device));
  lbm_solver *s = new (std::nothrow) lbm_solver();
  if (!s) return fail(LBM_ERR_ARG, "out of host memory");
  Ctx &c = s->c;
  c.cfg = *cfg;
  c.n = (int64_t)cfg->nx * cfg->ny * cfg->nz;
  c.gx = (cfg->nx + lbmk::BX - 1) / lbmk::BX;
  c.gy = (cfg->ny + lbmk::BY - 1) / lbmk::BY;
  c.nblocks = (int64_t)c.gx * c.gy * cfg->nz;
  c.odd_next = 1;
  c.omega_rot = cfg->omega_rot;
  {
    // the bulk-copy kernel moves 16-byte pieces: rows must split into them
    const int h = 16 / (int)storage_bytes(cfg->storage);
    const int tail = cfg->nx % lbmk::SW;
    c.use_stream = (cfg->flags & LBM_FLAG_BULKCOPY) && !(cfg->flags & LBM_FLAG_SIMT) && !cfg->heat && cfg->nx % h == 0 &&
                   cfg->nx >= 2 * h && (tail == 0 || tail >= 2 * h);
    c.wait_limit = lbmk::WAIT_LIMIT;
    c.starve_next = 0;
    c.nseg_x = (cfg->nx + lbmk::SW - 1) / lbmk::SW;
    c.nseg = c.nseg_x * cfg->ny * cfg->nz;
  }
  {
    // population layout: blocks of 32 cells with their 19 slots side by side
    // for the storage types that run faster so, where 32-bit offsets reach
    const int64_t nxb = (cfg->nx + lbmk::BLK - 1) / lbmk::BLK;
    c.npos = nxb * lbmk::BLK * cfg->ny * cfg->nz;
    c.rowp = (uint32_t)(nxb * lbmk::Q * lbmk::BLK);
    c.blocked = lbmk::blocked_layout((int)storage_bytes(cfg->storage)) && !c.use_stream &&
                !(cfg->flags & LBM_FLAG_SLOT_POINTERS) && 19 * c.npos <= (int64_t)UINT32_MAX;
  }
  {
    cudaError_t e0 = cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, cfg->device);
    if (e0 != cudaSuccess) {
      delete s;
      return fail(LBM_ERR_CUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e0));
    }
  }
  {
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    cudaError_t e0 = cudaStreamCreateWithPriority(&c.side, cudaStreamNonBlocking, hi);
    if (e0 == cudaSuccess) e0 = cudaStreamCreateWithFlags(&c.capture, cudaStreamNonBlocking);
    if (e0 == cudaSuccess) e0 = cudaEventCreateWithFlags(&c.fork, cudaEventDisableTiming);
    if (e0 == cudaSuccess) e0 = cudaEventCreateWithFlags(&c.join, cudaEventDisableTiming);
    if (e0 != cudaSuccess) {
      delete s;
      return fail(LBM_ERR_CUDA, std::string("side stream: ") + cudaGetErrorString(e0));
    }
  }
  auto bail = [&](lbm_status e) {
    release(s);
    delete s;
    return e;
  };
  const size_t fbytes = (size_t)19 * (size_t)(c.blocked ? c.npos : c.n) * storage_bytes(cfg->storage);
  cudaError_t e = cudaMalloc(&c.F, fbytes);
  if (e != cudaSuccess) return bail(fail(LBM_ERR_CUDA, std::string("population buffer: ") + cudaGetErrorString(e)));
  s->bytes += (int64_t)fbytes;
  for (int k = 0; k < LBM_NUM_FIELDS; ++k) {
    e = cudaMallocManaged(&c.fld[k], (size_t)c.n * sizeof(float), cudaMemAttachGlobal);
    if (e == cudaSuccess) place_on_device(c.fld[k], (size_t)c.n * sizeof(float), cfg->device);
    if (e == cudaSuccess) e = cudaMemset(c.fld[k], 0, (size_t)c.n * sizeof(float));
    if (e != cudaSuccess) return bail(fail(LBM_ERR_CUDA, std::string("cudaMallocManaged: ") + cudaGetErrorString(e)));
    s->bytes += c.n * (int64_t)sizeof(float);
  }
  c.nout = cfg->heat ? 6 : 5;
  if (cfg->heat) {
    const size_t gbytes = (size_t)7 * (size_t)c.n * sizeof(float);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
      e = cudaMalloc(&c.g[k], gbytes);
      if (e == cudaSuccess) e = cudaMemset(c.g[k], 0, gbytes);
    }
    if (e == cudaSuccess) e = cudaMalloc(&c.aux, (size_t)c.n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMemset(c.aux, 0, (size_t)c.n * sizeof(float4));
    for (int k = 0; k < LBM_NUM_HEAT_FIELDS && e == cudaSuccess; ++k) {
      e = cudaMallocManaged(&c.heat_fld[k], (size_t)c.n * sizeof(float), cudaMemAttachGlobal);
      if (e == cudaSuccess) place_on_device(c.heat_fld[k], (size_t)c.n * sizeof(float), cfg->device);
      if (e == cudaSuccess) e = cudaMemset(c.heat_fld[k], 0, (size_t)c.n * sizeof(float));
    }
    if (e != cudaSuccess) return bail(fail(LBM_ERR_CUDA, std::string("heat buffers: ") + cudaGetErrorString(e)));
    s->bytes += 2 * (int64_t)gbytes + c.n * (int64_t)(sizeof(float4) + LBM_NUM_HEAT_FIELDS * sizeof(float));
  }
  // fast-kernel blocks plus at most one general block per four warps
  c.partial_rows = std::max<int64_t>(2 * c.nblocks + 1, (int64_t)c.num_sms * 32);
  e = cudaMalloc(&c.fld_dev, LBM_NUM_FIELDS * sizeof(float *));
  if (e == cudaSuccess) e = cudaMemcpy(c.fld_dev, c.fld, LBM_NUM_FIELDS * sizeof(float *), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return bail(fail(LBM_ERR_CUDA, std::string("field table: ") + cudaGetErrorString(e)));
  e = cudaMalloc(&c.partials, (size_t)c.partial_rows * lbmk::NSUM * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&c.error, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemset(c.error, 0, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMalloc(&c.ticket, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMemset(c.ticket, 0, sizeof(unsigned int));
  if (e == cudaSuccess) e = cudaMalloc(&c.stage, lbmh::FINALIZE_BLOCKS * lbmk::NSUM * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&c.sums, lbmk::NSUM * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(c.sums, 0, lbmk::NSUM * sizeof(double));
  if (e != cudaSuccess) return bail(fail(LBM_ERR_CUDA, std::string("scratch: ") + cudaGetErrorString(e)));
  s->bytes += (c.partial_rows + lbmh::FINALIZE_BLOCKS + 1) * lbmk::NSUM * (int64_t)sizeof(double);
  st = set_reach(c);
  if (st != LBM_OK) return bail(st);
  st = classify_segments(s);
  if (st != LBM_OK) return bail(st);
  s->bytes += (int64_t)c.nseg * 4 + (int64_t)c.nmasked * (lbmk::SW + 1) * 4;
  release_output(c);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return bail(fail(LBM_ERR_CUDA, std::string("create: ") + cudaGetErrorString(e)));
  *out = s;
  return LBM_OK;
}

lbm_status lbm_destroy(lbm_solver *s) {
  if (!s) return LBM_OK;
  cudaSetDevice(s->c.cfg.device);
  cudaDeviceSynchronize();
  release(s);
  delete s;
  return LBM_OK;
}

#define LBM_HANDLE(s)                                        \
  do {                                                       \
    if (!(s)) return fail(LBM_ERR_ARG, "null solver handle"); \
    LBM_CUDA(cudaSetDevice((s)->c.cfg.device));              \
  } while (0)

lbm_status lbm_init(lbm_solver *s, double seed_amp) {
  lbmh::Range range_("lbm_init");
  LBM_HANDLE(s);
  if (!std::isfinite(seed_amp)) return fail(LBM_ERR_ARG, "seed_amp must be finite");
  s->c.odd_next = 1;
  LBM_CUDA(dispatch_init(s->c, seed_amp, 0));
  s->steps = 0;
  return LBM_OK;
}

lbm_status lbm_init_random(lbm_solver *s, double rho_sigma, double u_noise, uint64_t seed) {
  lbmh::Range range_("lbm_init_random");
  LBM_HANDLE(s);
  if (!std::isfinite(rho_sigma) || !std::isfinite(u_noise)) return fail(LBM_ERR_ARG, "non-finite noise");
  s->c.odd_next = 1;
  LBM_CUDA(dispatch_init_random(s->c, rho_sigma, u_noise, seed, 0));
  s->steps = 0;
  return LBM_OK;
}

lbm_status lbm_step(lbm_solver *s, int32_t report, void *stream) {
  lbmh::Range range_("lbm_step");
  LBM_HANDLE(s);
  const cudaError_t es = dispatch_step(s->c, report != 0, (cudaStream_t)stream);
  if (s->c.starve_next) {  // the stall test hook covers one step
    s->c.starve_next = 0;
    s->c.wait_limit = lbmk::WAIT_LIMIT;
  }
  LBM_CUDA(es);
  if (s->c.cfg.heat) {
    LBM_CUDA(lbmh::launch_heat(s->c, report != 0, (cudaStream_t)stream));
    s->c.g_cur ^= 1;
  }
  if (s->c.ev && s->c.ev_used < s->c.ev_cap) s->c.ev_used++;
  s->c.odd_next ^= 1;
  s->steps += 1;
  if (report) s->reported = true;
  return LBM_OK;
}

// One step's launches on `st` (the flow step, then the temperature step) and
// the bookkeeping that follows them.
static cudaError_t launch_one(lbm_solver *s, bool rep, cudaStream_t st) {
  Ctx &c = s->c;
  cudaError_t e = dispatch_step(c, rep, st);
  if (e == cudaSuccess && c.cfg.heat) {
    e = lbmh::launch_heat(c, rep, st);
    c.g_cur ^= 1;
  }
  c.odd_next ^= 1;
  return e;
}

// The graph of two quiet steps starting at parity c.odd_next, captured on the
// solver's capture stream the first time it is needed. Null when capture is
// not possible; the caller then launches the steps one by one.
static cudaGraphExec_t pair_graph(lbm_solver *s) {
  Ctx &c = s->c;
  cudaGraphExec_t &slot = c.pair_graph[c.odd_next];
  if (slot) return slot;
  if (cudaStreamBeginCapture(c.capture, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  const int odd = c.odd_next, g = c.g_cur;
  cudaError_t e = launch_one(s, false, c.capture);
  if (e == cudaSuccess) e = launch_one(s, false, c.capture);
  c.odd_next = odd;  // two flips: the same parity and temperature buffer again
  c.g_cur = g;
  cudaGraph_t graph = nullptr;
  const cudaError_t e2 = cudaStreamEndCapture(c.capture, &graph);
  if (e == cudaSuccess && e2 == cudaSuccess && graph) {
    if (cudaGraphInstantiate(&slot, graph, 0) != cudaSuccess) slot = nullptr;
  }
  if (graph) cudaGraphDestroy(graph);
  cudaGetLastError();
  return slot;
}

lbm_status lbm_run(lbm_solver *s, int32_t count, int32_t report_last, void *stream) {
  lbmh::Range range_("lbm_run");
  LBM_HANDLE(s);
  if (count < 0) return fail(LBM_ERR_ARG, "count must be >= 0");
  if (s->c.starve_next) return fail(LBM_ERR_STATE, "a stall test is pending: it applies to lbm_step only");
  const cudaStream_t st = (cudaStream_t)stream;
  const int32_t quiet = report_last ? count - 1 : count;
  int32_t k = 0;
  // pairs of quiet steps as graph launches (not while kernels are being timed)
  if (!s->c.ev && quiet >= 4) {
    while (quiet - k >= 2) {
      cudaGraphExec_t g = pair_graph(s);
      if (!g) break;
      LBM_CUDA(cudaGraphLaunch(g, st));
      s->steps += 2;
      k += 2;
    }
  }
  for (; k < count; ++k) {
    const bool rep = report_last && k == count - 1;
    LBM_CUDA(launch_one(s, rep, st));
    if (s->c.ev && s->c.ev_used < s->c.ev_cap) s->c.ev_used++;
    s->steps += 1;
    if (rep) s->reported = true;
  }
  return LBM_OK;
}

static lbm_status check_kernel_error(lbm_solver *s) {
  unsigned int flag = 0;
  LBM_CUDA(cudaDeviceSynchronize());
  if (!s->c.use_stream) return LBM_OK;  // only the bulk-copy kernel sets the flag
  LBM_CUDA(cudaMemcpy(&flag, s->c.error, sizeof(flag), cudaMemcpyDeviceToHost));
  if (flag) {
    cudaMemset(s->c.error, 0, sizeof(flag));
    return fail(LBM_ERR_CUDA, (flag & lbmk::STREAM_IN_FLIGHT)
                                  ? "a step kernel gave up waiting for its copies, and some were still "
                                    "unconfirmed when it ended; the populations are invalid"
                                  : "a step kernel gave up waiting for its copies; the populations are invalid");
  }
  return LBM_OK;
}

lbm_status lbm_field_sums(lbm_solver *s, double out[8]) {
  LBM_HANDLE(s);
  if (!out) return fail(LBM_ERR_ARG, "null output");
  lbm_status ks = check_kernel_error(s);
  if (ks != LBM_OK) return ks;
  LBM_CUDA(cudaMemcpy(out, s->c.sums, lbmk::NSUM * sizeof(double), cudaMemcpyDeviceToHost));
  return LBM_OK;
}

lbm_status lbm_monitors(lbm_solver *s, int32_t interval, double diameter, double out[7]) {
  lbmh::Range range_("lbm_monitors");
  if (!out) return fail(LBM_ERR_ARG, "null output");
  double t[8];
  lbm_status st = lbm_field_sums(s, t);
  if (st != LBM_OK) return st;
  const double n = (double)s->c.n;
  const double div = (double)std::max(interval, 1);
  for (int k = 0; k < 5; ++k) out[k] = std::sqrt(t[k] / n) / div;
  const double scale = 0.5 * s->c.cfg.u0 * s->c.cfg.u0 * diameter * s->c.cfg.nz;
  out[LBM_MON_DRAG] = t[5] / scale;
  out[LBM_MON_LIFT] = t[6] / scale;
  for (int k = 0; k < 7; ++k)
    if (!std::isfinite(out[k])) return fail(LBM_ERR_NONFINITE, "a monitor is not finite: the run diverged");
  return LBM_OK;
}

lbm_status lbm_field(lbm_solver *s, int32_t id, float **ptr) {
  if (!s || !ptr) return fail(LBM_ERR_ARG, "null argument");
  if (id < 0 || id >= LBM_NUM_FIELDS) return fail(LBM_ERR_ARG, "field id out of range");
  *ptr = s->c.fld[id];
  return LBM_OK;
}

lbm_status lbm_set_field(lbm_solver *s, int32_t id, const float *host) {
  LBM_HANDLE(s);
  if (!host || id < 0 || id >= LBM_NUM_FIELDS) return fail(LBM_ERR_ARG, "bad field id or null buffer");
  LBM_CUDA(cudaDeviceSynchronize());
  LBM_CUDA(cudaMemcpy(s->c.fld[id], host, (size_t)s->c.n * sizeof(float), cudaMemcpyDefault));
  return LBM_OK;
}

lbm_status lbm_set_physics(lbm_solver *s, int32_t collision, double nu, double cs) {
  if (!s) return fail(LBM_ERR_ARG, "null solver handle");
  lbm_config g = s->c.cfg;
  g.collision = collision;
  g.nu = nu;
  if (cs >= 0) g.cs = cs;
  lbm_status st = validate(g);
  if (st != LBM_OK) return st;
  s->c.cfg = g;
  drop_graphs(s->c);
  return LBM_OK;
}

lbm_status lbm_set_sponge(lbm_solver *s, double start, double strength) {
  if (!s) return fail(LBM_ERR_ARG, "null solver handle");
  if (!std::isfinite(start) || !std::isfinite(strength)) return fail(LBM_ERR_ARG, "non-finite sponge");
  s->c.cfg.sponge_start = start;
  s->c.cfg.sponge_strength = strength;
  drop_graphs(s->c);
  return LBM_OK;
}

lbm_status lbm_set_actuation(lbm_solver *s, double omega_rot) {
  if (!s) return fail(LBM_ERR_ARG, "null solver handle");
  if (!std::isfinite(omega_rot)) return fail(LBM_ERR_ARG, "non-finite rotation");
  if (omega_rot != s->c.omega_rot) drop_graphs(s->c);
  s->c.omega_rot = omega_rot;
  return LBM_OK;
}

lbm_status lbm_get_actuation(lbm_solver *s, double *omega_rot) {
  if (!s || !omega_rot) return fail(LBM_ERR_ARG, "null argument");
  *omega_rot = s->c.omega_rot;
  return LBM_OK;
}

static lbm_status copy_in(lbm_solver *s, const void *f, int32_t dtype, int32_t where) {
  const size_t bytes = (size_t)19 * (size_t)s->c.n * (dtype == LBM_F64 ? 8 : 4);
  if (where == LBM_DEVICE) {
    LBM_CUDA(dispatch_import(s->c, f, dtype, 0));
    LBM_CUDA(cudaDeviceSynchronize());
    return LBM_OK;
  }
  void *tmp = nullptr;
  LBM_CUDA(cudaMalloc(&tmp, bytes));
  cudaError_t e = cudaMemcpy(tmp, f, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = dispatch_import(s->c, tmp, dtype, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  cudaFree(tmp);
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("set_populations: ") + cudaGetErrorString(e));
  return LBM_OK;
}

static lbm_status copy_out(lbm_solver *s, void *f, int32_t dtype, int32_t where) {
  const size_t bytes = (size_t)19 * (size_t)s->c.n * (dtype == LBM_F64 ? 8 : 4);
  if (where == LBM_DEVICE) {
    LBM_CUDA(dispatch_export(s->c, f, dtype, 0));
    LBM_CUDA(cudaDeviceSynchronize());
    return LBM_OK;
  }
  void *tmp = nullptr;
  LBM_CUDA(cudaMalloc(&tmp, bytes));
  cudaError_t e = dispatch_export(s->c, tmp, dtype, 0);
  if (e == cudaSuccess) e = cudaMemcpy(f, tmp, bytes, cudaMemcpyDeviceToHost);
  cudaFree(tmp);
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("get_populations: ") + cudaGetErrorString(e));
  return LBM_OK;
}

lbm_status lbm_set_populations(lbm_solver *s, const void *f, int32_t dtype, int32_t where) {
  LBM_HANDLE(s);
  if (!f || (dtype != LBM_F32 && dtype != LBM_F64) || (where != LBM_HOST && where != LBM_DEVICE))
    return fail(LBM_ERR_ARG, "bad populations buffer, dtype or location");
  LBM_CUDA(cudaDeviceSynchronize());
  s->c.odd_next = 1;
  s->steps = 0;
  return copy_in(s, f, dtype, where);
}

lbm_status lbm_get_populations(lbm_solver *s, void *f, int32_t dtype, int32_t where) {
  LBM_HANDLE(s);
  if (!f || (dtype != LBM_F32 && dtype != LBM_F64) || (where != LBM_HOST && where != LBM_DEVICE))
    return fail(LBM_ERR_ARG, "bad populations buffer, dtype or location");
  LBM_CUDA(cudaDeviceSynchronize());
  return copy_out(s, f, dtype, where);
}

lbm_status lbm_set_obstacle(lbm_solver *s, int32_t kind, const double geo[7]) {
  LBM_HANDLE(s);
  if (!geo) return fail(LBM_ERR_ARG, "null geometry");
  lbm_config g = s->c.cfg;
  g.obstacle = kind;
  g.ox = geo[0];
  g.oy = geo[1];
  g.oz = geo[2];
  g.r = geo[3];
  g.hx = geo[4];
  g.hy = geo[5];
  g.hz = geo[6];
  lbm_status st = validate(g);
  if (st != LBM_OK) return st;
  // carry the populations over: read them out with the old geometry, write them
  // back (start-of-step layout) with the new one
  const int dtype = g.storage == LBM_F64 ? LBM_F64 : LBM_F32;
  const size_t bytes = (size_t)19 * (size_t)s->c.n * (dtype == LBM_F64 ? 8 : 4);
  void *tmp = nullptr;
  LBM_CUDA(cudaDeviceSynchronize());
  LBM_CUDA(cudaMalloc(&tmp, bytes));
  cudaError_t e = dispatch_export(s->c, tmp, dtype, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    cudaFree(tmp);
    return fail(LBM_ERR_CUDA, std::string("set_obstacle: ") + cudaGetErrorString(e));
  }
  s->c.cfg = g;
  drop_graphs(s->c);
  st = set_reach(s->c);
  if (st == LBM_OK) st = classify_segments(s);
  if (st == LBM_OK) {
    s->c.odd_next = 1;
    e = dispatch_import(s->c, tmp, dtype, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) st = fail(LBM_ERR_CUDA, std::string("set_obstacle: ") + cudaGetErrorString(e));
  }
  cudaFree(tmp);
  return st;
}

lbm_status lbm_set_output_stride(lbm_solver *s, int32_t stride) {
  LBM_HANDLE(s);
  if (stride < 1) return fail(LBM_ERR_ARG, "stride must be >= 1");
  LBM_CUDA(cudaDeviceSynchronize());
  Ctx &c = s->c;
  release_output(c);
  if (stride == 1) return LBM_OK;
  const int dims[3] = {c.cfg.nx, c.cfg.ny, c.cfg.nz};
  size_t m = 1;
  for (int k = 0; k < 3; ++k) {
    c.out_dims[k] = (dims[k] + stride - 1) / stride;
    m *= (size_t)c.out_dims[k];
  }
  for (int k = 0; k < c.nout; ++k) {
    c.out[k] = nullptr;
    cudaError_t e = cudaMallocManaged(&c.out[k], m * sizeof(float), cudaMemAttachGlobal);
    if (e == cudaSuccess) place_on_device(c.out[k], m * sizeof(float), c.cfg.device);
    if (e != cudaSuccess) {
      for (int j = 0; j < k; ++j) cudaFree(c.out[j]);
      for (int j = 0; j < c.nout; ++j) c.out[j] = lbmh::output_source(c, j);
      c.out_dims[0] = c.cfg.nx;
      c.out_dims[1] = c.cfg.ny;
      c.out_dims[2] = c.cfg.nz;
      return fail(LBM_ERR_CUDA, std::string("output fields: ") + cudaGetErrorString(e));
    }
    cudaMemset(c.out[k], 0, m * sizeof(float));
  }
  LBM_CUDA(cudaDeviceSynchronize());
  c.out_stride = stride;
  return LBM_OK;
}

lbm_status lbm_output(lbm_solver *s, int32_t id, float **ptr, int64_t *count) {
  if (!s || !ptr || !count) return fail(LBM_ERR_ARG, "null argument");
  if (id < 0 || id >= s->c.nout)
    return fail(LBM_ERR_ARG, "output id out of range (ux, uy, uz, p, vmag; temp with heat)");
  *ptr = s->c.out[id];
  *count = (int64_t)s->c.out_dims[0] * s->c.out_dims[1] * s->c.out_dims[2];
  return LBM_OK;
}

lbm_status lbm_update_output(lbm_solver *s, void *stream) {
  lbmh::Range range_("lbm_update_output");
  LBM_HANDLE(s);
  LBM_CUDA(lbmh::launch_coarsen(s->c, (cudaStream_t)stream));
  return LBM_OK;
}

lbm_status lbm_mask(lbm_solver *s, uint8_t *host_out) {
  LBM_HANDLE(s);
  if (!host_out) return fail(LBM_ERR_ARG, "null output");
  uint8_t *tmp = nullptr;
  LBM_CUDA(cudaMalloc(&tmp, (size_t)s->c.n));
  cudaError_t e = lbmh::launch_mask(s->c, tmp, 0);
  if (e == cudaSuccess) e = cudaMemcpy(host_out, tmp, (size_t)s->c.n, cudaMemcpyDeviceToHost);
  cudaFree(tmp);
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("mask: ") + cudaGetErrorString(e));
  return LBM_OK;
}

lbm_status lbm_step_count(lbm_solver *s, int64_t *count) {
  if (!s || !count) return fail(LBM_ERR_ARG, "null argument");
  *count = s->steps;
  return LBM_OK;
}

lbm_status lbm_memory(lbm_solver *s, int64_t *bytes) {
  if (!s || !bytes) return fail(LBM_ERR_ARG, "null argument");
  *bytes = s->bytes;
  return LBM_OK;
}

lbm_status lbm_managed_alloc(int64_t count, float **ptr) {
  if (!ptr || count < 1) return fail(LBM_ERR_ARG, "count must be >= 1 and ptr non-null");
  *ptr = nullptr;
  LBM_CUDA(cudaMallocManaged(ptr, (size_t)count * sizeof(float), cudaMemAttachGlobal));
  LBM_CUDA(cudaMemset(*ptr, 0, (size_t)count * sizeof(float)));
  LBM_CUDA(cudaDeviceSynchronize());
  return LBM_OK;
}

lbm_status lbm_managed_free(float *ptr) {
  if (ptr) LBM_CUDA(cudaFree(ptr));
  return LBM_OK;
}

lbm_status lbm_timing(lbm_solver *s, int32_t enable) {
  LBM_HANDLE(s);
  LBM_CUDA(cudaDeviceSynchronize());
  Ctx &c = s->c;
  release_timing(c);
  if (!enable) return LBM_OK;
  const int cap = 4096;
  c.ev = new (std::nothrow) cudaEvent_t[3 * cap];
  if (!c.ev) return fail(LBM_ERR_ARG, "out of host memory");
  for (int k = 0; k < 3 * cap; ++k) {
    cudaError_t e = cudaEventCreate(&c.ev[k]);
    if (e != cudaSuccess) {
      for (int j = 0; j < k; ++j) cudaEventDestroy(c.ev[j]);
      delete[] c.ev;
      c.ev = nullptr;
      return fail(LBM_ERR_CUDA, std::string("cudaEventCreate: ") + cudaGetErrorString(e));
    }
  }
  c.ev_cap = cap;
  c.ev_used = 0;
  c.generic_cells = c.use_stream ? 0 : c.special_cells;
  c.bulk_cells = c.n - c.generic_cells;  // the dominant kernel's cells
  return LBM_OK;
}

lbm_status lbm_timing_read(lbm_solver *s, double out[7]) {
  LBM_HANDLE(s);
  if (!out) return fail(LBM_ERR_ARG, "null output");
  LBM_CUDA(cudaDeviceSynchronize());
  const Ctx &c = s->c;
  double bulk = 0.0, gen = 0.0;
  for (int k = 0; k < c.ev_used; ++k) {
    float a = 0.f, b = 0.f;
    LBM_CUDA(cudaEventElapsedTime(&a, c.ev[3 * k], c.ev[3 * k + 1]));
    LBM_CUDA(cudaEventElapsedTime(&b, c.ev[3 * k + 1], c.ev[3 * k + 2]));
    bulk += a;
    gen += b;
  }
  float span = 0.f;
  if (c.ev_used > 0) LBM_CUDA(cudaEventElapsedTime(&span, c.ev[0], c.ev[3 * (c.ev_used - 1) + 2]));
  out[6] = span;
  out[0] = bulk;
  out[1] = c.ev_used;
  out[2] = (double)c.bulk_cells;
  out[3] = gen;
  out[4] = c.ev_used;
  out[5] = (double)c.generic_cells;
  return LBM_OK;
}

lbm_status lbm_sync(lbm_solver *s) {
  LBM_HANDLE(s);
  return check_kernel_error(s);
}

lbm_status lbm_test_bulkcopy_stall(lbm_solver *s, int64_t wait_polls) {
  LBM_HANDLE(s);
  if (!s->c.use_stream) return fail(LBM_ERR_STATE, "the solver does not use the bulk-copy kernel");
  if (wait_polls < 1) return fail(LBM_ERR_ARG, "wait_polls must be >= 1");
  s->c.starve_next = 1;
  s->c.wait_limit = wait_polls;
  return LBM_OK;
}

lbm_status lbm_heat_field(lbm_solver *s, int32_t id, float **ptr) {
  if (!s || !ptr) return fail(LBM_ERR_ARG, "null argument");
  if (!s->c.cfg.heat) return fail(LBM_ERR_STATE, "the run has no heat");
  if (id < 0 || id >= LBM_NUM_HEAT_FIELDS) return fail(LBM_ERR_ARG, "heat field id out of range (t_solid, q_solid, temp)");
  *ptr = s->c.heat_fld[id];
  return LBM_OK;
}

static lbm_status heat_copy(lbm_solver *s, void *host, int32_t dtype, int32_t where, bool in) {
  if (!s || !host) return fail(LBM_ERR_ARG, "null argument");
  if (!s->c.cfg.heat) return fail(LBM_ERR_STATE, "the run has no heat");
  if (dtype != LBM_F32 && dtype != LBM_F64) return fail(LBM_ERR_ARG, "dtype must be LBM_F32 or LBM_F64");
  if (where != LBM_HOST && where != LBM_DEVICE) return fail(LBM_ERR_ARG, "where must be LBM_HOST or LBM_DEVICE");
  LBM_CUDA(cudaSetDevice(s->c.cfg.device));
  LBM_CUDA(cudaDeviceSynchronize());
  const size_t m = (size_t)7 * (size_t)s->c.n;
  float *dev = s->c.g[s->c.g_cur];
  if (dtype == LBM_F32) {
    const cudaMemcpyKind kind = in ? (where == LBM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice)
                                   : (where == LBM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice);
    LBM_CUDA(in ? cudaMemcpy(dev, host, m * sizeof(float), kind) : cudaMemcpy(host, dev, m * sizeof(float), kind));
    return LBM_OK;
  }
  // float64 values: converted on the host
  std::vector<double> d(m);
  std::vector<float> f(m);
  if (in) {
    LBM_CUDA(cudaMemcpy(d.data(), host, m * sizeof(double),
                        where == LBM_HOST ? cudaMemcpyHostToHost : cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < m; ++i) f[i] = (float)d[i];
    LBM_CUDA(cudaMemcpy(dev, f.data(), m * sizeof(float), cudaMemcpyHostToDevice));
  } else {
    LBM_CUDA(cudaMemcpy(f.data(), dev, m * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < m; ++i) d[i] = (double)f[i];
    LBM_CUDA(cudaMemcpy(host, d.data(), m * sizeof(double),
                        where == LBM_HOST ? cudaMemcpyHostToHost : cudaMemcpyHostToDevice));
  }
  return LBM_OK;
}

lbm_status lbm_set_heat_populations(lbm_solver *s, const void *g, int32_t dtype, int32_t where) {
  return heat_copy(s, const_cast<void *>(g), dtype, where, true);
}

lbm_status lbm_get_heat_populations(lbm_solver *s, void *g, int32_t dtype, int32_t where) {
  return heat_copy(s, g, dtype, where, false);
}

lbm_status lbm_set_sink(lbm_solver *s, const double sink[8]) {
  LBM_HANDLE(s);
  if (!sink) return fail(LBM_ERR_ARG, "null sink");
  lbm_config g = s->c.cfg;
  for (int k = 0; k < 8; ++k) g.sink[k] = sink[k];
  if (g.obstacle != LBM_HEATSINK) {
    g.obstacle = LBM_HEATSINK;  // validate the sizes as a heat sink
    lbm_status st = validate(g);
    if (st != LBM_OK) return st;
    for (int k = 0; k < 8; ++k) s->c.cfg.sink[k] = sink[k];
    drop_graphs(s->c);
    return LBM_OK;
  }
  double geo[7] = {g.ox, g.oy, g.oz, g.r, g.hx, g.hy, g.hz};
  for (int k = 0; k < 8; ++k) s->c.cfg.sink[k] = sink[k];
  drop_graphs(s->c);
  return lbm_set_obstacle(s, LBM_HEATSINK, geo);
}

lbm_status lbm_read_output(lbm_solver *s, int32_t id, float *host, void *stream) {
  lbmh::Range range_("lbm_read_output");
  LBM_HANDLE(s);
  if (!host) return fail(LBM_ERR_ARG, "null host buffer");
  if (id < 0 || id >= s->c.nout)
    return fail(LBM_ERR_ARG, "output id out of range (ux, uy, uz, p, vmag; temp with heat)");
  const size_t m = (size_t)s->c.out_dims[0] * s->c.out_dims[1] * s->c.out_dims[2];
  LBM_CUDA(cudaMemcpyAsync(host, s->c.out[id], m * sizeof(float), cudaMemcpyDefault, (cudaStream_t)stream));
  return LBM_OK;
}

lbm_status lbm_velocity_gradient(lbm_solver *s, float *jac, double inv_h, void *stream) {
  lbmh::Range range_("lbm_velocity_gradient");
  LBM_HANDLE(s);
  if (!jac) return fail(LBM_ERR_ARG, "null gradient buffer");
  if (!std::isfinite(inv_h)) return fail(LBM_ERR_ARG, "inv_h must be finite");
  LBM_CUDA(lbmh::launch_jacobian(s->c, jac, (float)inv_h, (cudaStream_t)stream));
  return LBM_OK;
}

lbm_status lbm_vorticity_q(lbm_solver *s, const float *jac, float *vorticity, float *q, int32_t at_cells,
                           void *stream) {
  lbmh::Range range_("lbm_vorticity_q");
  LBM_HANDLE(s);
  if (!jac) return fail(LBM_ERR_ARG, "null gradient buffer");
  if (at_cells != 0 && at_cells != 1) return fail(LBM_ERR_ARG, "at_cells must be 0 or 1");
  LBM_CUDA(lbmh::launch_vortq(s->c, jac, vorticity, q, at_cells, (cudaStream_t)stream));
  return LBM_OK;
}

lbm_status lbm_vorticity_q_direct(lbm_solver *s, double inv_h, float *vorticity, float *q, int32_t at_cells,
                                  void *stream) {
  lbmh::Range range_("lbm_vorticity_q_direct");
  LBM_HANDLE(s);
  if (!std::isfinite(inv_h)) return fail(LBM_ERR_ARG, "inv_h must be finite");
  if (at_cells != 0 && at_cells != 1) return fail(LBM_ERR_ARG, "at_cells must be 0 or 1");
  LBM_CUDA(lbmh::launch_vortq_direct(s->c, (float)inv_h, vorticity, q, at_cells, (cudaStream_t)stream));
  return LBM_OK;
}

lbm_status lbm_run_timed(lbm_solver *s, int32_t count, int32_t report_last, void *stream, double *ms) {
  lbmh::Range range_("lbm_run_timed");
  LBM_HANDLE(s);
  if (!ms) return fail(LBM_ERR_ARG, "null output");
  cudaEvent_t ev[2] = {nullptr, nullptr};
  LBM_CUDA(cudaEventCreate(&ev[0]));
  cudaError_t e = cudaEventCreate(&ev[1]);
  if (e == cudaSuccess) e = cudaEventRecord(ev[0], (cudaStream_t)stream);
  lbm_status st = e == cudaSuccess ? lbm_run(s, count, report_last, stream) : LBM_ERR_CUDA;
  if (st == LBM_OK) {
    e = cudaEventRecord(ev[1], (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, ev[0], ev[1]);
    *ms = t;
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (st != LBM_OK) return st;
  if (e != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("lbm_run_timed: ") + cudaGetErrorString(e));
  return LBM_OK;
}

}  // extern "C"
