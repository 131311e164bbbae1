// lbm_derived.cu - velocity gradient, vorticity and Q-criterion on the output grid.
//
// The solver side of tack-lbm's derived fields (derived.py): the velocity
// gradient on the (coarsened) output grid by central differences, one-sided
// at the grid's faces, in units of the spacing h = stride / diameter
// (derived.py:52-89, 101-103), and the two default derived fields computed
// from it, |curl u| and Q = -1/2 sum_ij J_ij J_ji (derived.py:27-30).
// At points they use the point's gradient; at cell centres the mean of the
// gradients at the cell's eight corners (the trilinear interpolant at the
// centre).
#include <cuda_runtime.h>

#include "lbm_device.cuh"
#include "lbm_host.h"

namespace {

struct Vel {
  const float *u[3];
};

// g[3 c + d] = d u_c / d x_d at output point (i, j, k) (derived.py:57-89):
// central differences, one-sided at the grid's faces, times 1/h. Each entry
// is one rounded difference times one rounded scale (no fused multiply-add),
// so every kernel below computes the same float for the same point.
__device__ __forceinline__ void point_gradient(const Vel &v, int i, int j, int k, int mx, int my, int mz,
                                               float inv_h, float g[9]) {
  const int xl = i > 0 ? i - 1 : i, xh = i < mx - 1 ? i + 1 : i;
  const int yl = j > 0 ? j - 1 : j, yh = j < my - 1 ? j + 1 : j;
  const int zl = k > 0 ? k - 1 : k, zh = k < mz - 1 ? k + 1 : k;
  const float sx = xh > xl ? inv_h / (float)(xh - xl) : 0.f;
  const float sy = yh > yl ? inv_h / (float)(yh - yl) : 0.f;
  const float sz = zh > zl ? inv_h / (float)(zh - zl) : 0.f;
  const int base = mx * (j + my * k);
  const int x0 = xl + base, x1 = xh + base;
  const int y0 = i + mx * (yl + my * k), y1 = i + mx * (yh + my * k);
  const int z0 = i + mx * (j + my * zl), z1 = i + mx * (j + my * zh);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float *u = v.u[c];
    g[3 * c + 0] = __fmul_rn(__fsub_rn(__ldg(u + x1), __ldg(u + x0)), sx);
    g[3 * c + 1] = __fmul_rn(__fsub_rn(__ldg(u + y1), __ldg(u + y0)), sy);
    g[3 * c + 2] = __fmul_rn(__fsub_rn(__ldg(u + z1), __ldg(u + z0)), sz);
  }
}

// jac[9 p + 3 c + d] = d u_c / d x_d at output point p. A block's 256 points
// go through shared memory, so the 9-float rows leave as coalesced stores.
constexpr int JAC_THREADS = 256;
__global__ void __launch_bounds__(JAC_THREADS)
jacobian_kernel(Vel v, float *jac, int mx, int my, int mz, float inv_h) {
  __shared__ float rows[9 * JAC_THREADS];
  const int m = mx * my * mz;
  for (int p0 = blockIdx.x * JAC_THREADS; p0 < m; p0 += gridDim.x * JAC_THREADS) {
    const int p = p0 + (int)threadIdx.x;
    if (p < m) {
      float g[9];
      point_gradient(v, p % mx, (p / mx) % my, p / (mx * my), mx, my, mz, inv_h, g);
#pragma unroll
      for (int e = 0; e < 9; ++e) rows[9 * threadIdx.x + e] = g[e];
    }
    __syncthreads();
    const int count = 9 * min(JAC_THREADS, m - p0);
    for (int t = (int)threadIdx.x; t < count; t += JAC_THREADS) jac[(size_t)9 * p0 + t] = rows[t];
    __syncthreads();
  }
}

__device__ __forceinline__ void vort_q(const float g[9], float &vort, float &q) {
  const float wx = g[7] - g[5], wy = g[2] - g[6], wz = g[3] - g[1];
  vort = sqrtf(wx * wx + wy * wy + wz * wz);
  float s = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) s += g[3 * a + b] * g[3 * b + a];
  q = -0.5f * s;
}

// |curl u| and Q straight from the velocity, without a gradient buffer, at
// the output points: each point's gradient where it is used.
__global__ void vortq_points_kernel(Vel v, float *vort, float *qc, int mx, int my, int mz, float inv_h) {
  const int m = mx * my * mz;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < m; p += gridDim.x * blockDim.x) {
    float g[9];
    point_gradient(v, p % mx, (p / mx) % my, p / (mx * my), mx, my, mz, inv_h, g);
    float w, q;
    vort_q(g, w, q);
    if (vort) vort[p] = w;
    if (qc) qc[p] = q;
  }
}

// The same at cell centres. A block takes a tile of CTX x CTY x CTZ cells:
// the gradients of the tile's (CTX+1)(CTY+1)(CTZ+1) corner points go to
// shared memory once, then each cell adds its eight corners in the order
// c = 0..7 that vortq_kernel uses, so the results equal the two-pass path's.
constexpr int CTX = 32, CTY = 4, CTZ = 2, CT = CTX * CTY * CTZ;
constexpr int PTX = CTX + 1, PTY = CTY + 1, PTZ = CTZ + 1, PT = PTX * PTY * PTZ;
__global__ void __launch_bounds__(CT) vortq_cells_kernel(Vel v, float *vort, float *qc, int mx, int my, int mz,
                                                        float inv_h) {
  __shared__ float gs[9 * PT];
  const int i0 = (int)blockIdx.x * CTX, j0 = (int)blockIdx.y * CTY, k0 = (int)blockIdx.z * CTZ;
  for (int t = (int)threadIdx.x; t < PT; t += CT) {
    const int i = i0 + t % PTX, j = j0 + (t / PTX) % PTY, k = k0 + t / (PTX * PTY);
    if (i < mx && j < my && k < mz) {
      float g[9];
      point_gradient(v, i, j, k, mx, my, mz, inv_h, g);
#pragma unroll
      for (int e = 0; e < 9; ++e) gs[9 * t + e] = g[e];
    }
  }
  __syncthreads();
  const int ti = (int)threadIdx.x % CTX, tj = ((int)threadIdx.x / CTX) % CTY, tk = (int)threadIdx.x / (CTX * CTY);
  const int i = i0 + ti, j = j0 + tj, k = k0 + tk;
  const int cx = mx - 1, cy = my - 1, cz = mz - 1;
  if (i >= cx || j >= cy || k >= cz) return;
  float g[9];
#pragma unroll
  for (int e = 0; e < 9; ++e) g[e] = 0.f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int t = (ti + (c & 1)) + PTX * ((tj + ((c >> 1) & 1)) + PTY * (tk + (c >> 2)));
#pragma unroll
    for (int e = 0; e < 9; ++e) g[e] = __fadd_rn(g[e], gs[9 * t + e]);
  }
#pragma unroll
  for (int e = 0; e < 9; ++e) g[e] *= 0.125f;
  float w, q;
  vort_q(g, w, q);
  const int p = i + cx * (j + cy * k);
  if (vort) vort[p] = w;
  if (qc) qc[p] = q;
}

// at_cells = 0: one value per point; 1: one per cell (mx-1)(my-1)(mz-1)
__global__ void vortq_kernel(const float *jac, float *vort, float *qc, int mx, int my, int mz, int at_cells) {
  const int cx = at_cells ? mx - 1 : mx, cy = at_cells ? my - 1 : my, cz = at_cells ? mz - 1 : mz;
  const int m = cx * cy * cz;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < m; p += gridDim.x * blockDim.x) {
    float g[9];
    if (!at_cells) {
#pragma unroll
      for (int e = 0; e < 9; ++e) g[e] = jac[(size_t)9 * p + e];
    } else {
      const int i = p % cx, j = (p / cx) % cy, k = p / (cx * cy);
#pragma unroll
      for (int e = 0; e < 9; ++e) g[e] = 0.f;
      for (int c = 0; c < 8; ++c) {
        const int pt = (i + (c & 1)) + mx * ((j + ((c >> 1) & 1)) + my * (k + (c >> 2)));
#pragma unroll
        for (int e = 0; e < 9; ++e) g[e] = __fadd_rn(g[e], jac[(size_t)9 * pt + e]);
      }
#pragma unroll
      for (int e = 0; e < 9; ++e) g[e] *= 0.125f;
    }
    float v, q;
    vort_q(g, v, q);
    if (vort) vort[p] = v;
    if (qc) qc[p] = q;
  }
}

}  // namespace

namespace lbmh {

cudaError_t launch_jacobian(const Ctx &c, float *jac, float inv_h, cudaStream_t st) {
  const int m = c.out_dims[0] * c.out_dims[1] * c.out_dims[2];
  const Vel v{{c.out[0], c.out[1], c.out[2]}};
  jacobian_kernel<<<lbmk::cell_grid(m), JAC_THREADS, 0, st>>>(v, jac, c.out_dims[0], c.out_dims[1],
                                                               c.out_dims[2], inv_h);
  return cudaGetLastError();
}

cudaError_t launch_vortq_direct(const Ctx &c, float inv_h, float *vort, float *q, int at_cells,
                                cudaStream_t st) {
  const int mx = c.out_dims[0], my = c.out_dims[1], mz = c.out_dims[2];
  const Vel v{{c.out[0], c.out[1], c.out[2]}};
  if (!at_cells) {
    vortq_points_kernel<<<lbmk::cell_grid((long long)mx * my * mz), 256, 0, st>>>(v, vort, q, mx, my, mz, inv_h);
  } else if (mx > 1 && my > 1 && mz > 1) {
    const dim3 grid((mx - 1 + CTX - 1) / CTX, (my - 1 + CTY - 1) / CTY, (mz - 1 + CTZ - 1) / CTZ);
    vortq_cells_kernel<<<grid, CT, 0, st>>>(v, vort, q, mx, my, mz, inv_h);
  }
  return cudaGetLastError();
}

cudaError_t launch_vortq(const Ctx &c, const float *jac, float *vort, float *q, int at_cells, cudaStream_t st) {
  const int m = c.out_dims[0] * c.out_dims[1] * c.out_dims[2];
  vortq_kernel<<<lbmk::cell_grid(m), 256, 0, st>>>(jac, vort, q, c.out_dims[0], c.out_dims[1], c.out_dims[2],
                                                   at_cells);
  return cudaGetLastError();
}

}  // namespace lbmh
