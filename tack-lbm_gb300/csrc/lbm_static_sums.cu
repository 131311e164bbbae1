// lbm_static_sums.cu - the monitor sums of caller-owned fields, with no allocation.
//
// Some callers cannot allocate device memory while the solver runs: an
// in-situ pipeline or host framework that owns every device buffer itself
// (it hands over preallocated fields and forbids allocation mid-run, because
// cudaMalloc synchronises the device and can fail under memory pressure), or a
// deployment that must keep a fixed device footprint. lbm_field_sums_static
// gives them the FP64 sums that Solver.monitors needs without any allocation:
// the caller passes the eight report fields and the output, and the per-block
// partial sums go to the fixed scratch array below.
//
// The scratch is a file-scope __device__ array of MAX_BLOCKS (16384) x 8
// doubles (1 MiB), one partial per 16384 cells, hence at most 2^28 cells. Every GPU that loads this library holds it until the
// process exits. All calls share it: two calls whose kernels overlap on the
// GPU (different streams, or different host threads on one device) race on
// it. Nothing in it needs clearing between calls: each call's first kernel
// writes every slot its second kernel reads.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "lbm_host.h"

namespace {

constexpr int SUMS = 8;
constexpr int THREADS = 256;
constexpr int64_t CELLS_PER_BLOCK = 16384;
constexpr int MAX_BLOCKS = 16384;  // LBM_STATIC_SUMS_MAX_CELLS / CELLS_PER_BLOCK
static_assert((int64_t)MAX_BLOCKS * CELLS_PER_BLOCK == LBM_STATIC_SUMS_MAX_CELLS, "limit mismatch");

static __device__ __align__(256) double g_partials[MAX_BLOCKS * SUMS];

// Per-device device address of g_partials, looked up once per device.
constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
double *g_ptr[MAX_DEVICES] = {};

struct Fields8 {
  const float *f[SUMS];
};

// Block b sums cells [b*CELLS_PER_BLOCK, (b+1)*CELLS_PER_BLOCK) of each field in FP64.
__global__ void __launch_bounds__(THREADS) partial_sums(Fields8 in, int64_t n, double *partials) {
  __shared__ double red[THREADS / 32][SUMS];
  const int64_t begin = (int64_t)blockIdx.x * CELLS_PER_BLOCK;
  const int64_t end = begin + CELLS_PER_BLOCK < n ? begin + CELLS_PER_BLOCK : n;
  double acc[SUMS];
#pragma unroll
  for (int k = 0; k < SUMS; ++k) acc[k] = 0.0;
  for (int64_t i = begin + threadIdx.x; i < end; i += THREADS) {
#pragma unroll
    for (int k = 0; k < SUMS; ++k) acc[k] += (double)in.f[k][i];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < SUMS; ++k) {
    double s = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) red[warp][k] = s;
  }
  __syncthreads();
  if (threadIdx.x < SUMS) {
    double s = 0.0;
    for (int w = 0; w < THREADS / 32; ++w) s += red[w][threadIdx.x];
    partials[(int64_t)blockIdx.x * SUMS + threadIdx.x] = s;
  }
}

// One block: the partials of `blocks` blocks, summed in a fixed order.
__global__ void __launch_bounds__(THREADS) final_sums(const double *partials, int blocks, double *sums) {
  __shared__ double red[THREADS][SUMS];
  double acc[SUMS];
#pragma unroll
  for (int k = 0; k < SUMS; ++k) acc[k] = 0.0;
  for (int b = threadIdx.x; b < blocks; b += THREADS) {
#pragma unroll
    for (int k = 0; k < SUMS; ++k) acc[k] += partials[(int64_t)b * SUMS + k];
  }
#pragma unroll
  for (int k = 0; k < SUMS; ++k) red[threadIdx.x][k] = acc[k];
  __syncthreads();
  for (int w = THREADS / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
#pragma unroll
      for (int k = 0; k < SUMS; ++k) red[threadIdx.x][k] += red[threadIdx.x + w][k];
    __syncthreads();
  }
  if (threadIdx.x < SUMS) sums[threadIdx.x] = red[0][threadIdx.x];
}

lbm_status static_fail(lbm_status s, const std::string &msg) {
  lbmh::set_last_error(msg);
  return s;
}

}  // namespace

extern "C" {

lbm_status lbm_field_sums_static(const float *const fields[8], int64_t n, double *sums, void *stream) {
  if (!fields || !sums) return static_fail(LBM_ERR_ARG, "fields and sums must be non-null");
  for (int k = 0; k < SUMS; ++k)
    if (!fields[k]) return static_fail(LBM_ERR_ARG, "every field pointer must be non-null");
  if (n < 1 || n > LBM_STATIC_SUMS_MAX_CELLS)
    return static_fail(LBM_ERR_ARG, "n must be in [1, LBM_STATIC_SUMS_MAX_CELLS = 2^28] cells; "
                                    "larger fields need lbm_field_sums on a solver");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return static_fail(LBM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= MAX_DEVICES) return static_fail(LBM_ERR_ARG, "device ordinal above 63");
  double *scratch = nullptr;
  {
    // set-up, once per device, with that device current
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_ptr[dev]) {
      e = cudaGetSymbolAddress((void **)&g_ptr[dev], g_partials);
      if (e != cudaSuccess) {
        g_ptr[dev] = nullptr;
        return static_fail(LBM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      }
    }
    scratch = g_ptr[dev];
  }
  Fields8 in;
  for (int k = 0; k < SUMS; ++k) in.f[k] = fields[k];
  const int blocks = (int)((n + CELLS_PER_BLOCK - 1) / CELLS_PER_BLOCK);
  cudaStream_t st = (cudaStream_t)stream;
  partial_sums<<<blocks, THREADS, 0, st>>>(in, n, scratch);
  final_sums<<<1, THREADS, 0, st>>>(scratch, blocks, sums);
  e = cudaGetLastError();
  if (e != cudaSuccess) return static_fail(LBM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return LBM_OK;
}

}  // extern "C"
