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

// jac[9 p + 3 c + d] = d u_c / d x_d at output point p (derived.py:57-89)
__global__ void jacobian_kernel(const float *ux, const float *uy, const float *uz, float *jac, int mx, int my,
                                int mz, float inv_h) {
  const int m = mx * my * mz;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < m; p += gridDim.x * blockDim.x) {
    const int i = p % mx, j = (p / mx) % my, k = p / (mx * my);
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
    const float *u[3] = {ux, uy, uz};
    float *o = jac + (size_t)9 * p;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      o[3 * c + 0] = (u[c][x1] - u[c][x0]) * sx;
      o[3 * c + 1] = (u[c][y1] - u[c][y0]) * sy;
      o[3 * c + 2] = (u[c][z1] - u[c][z0]) * sz;
    }
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
        for (int e = 0; e < 9; ++e) g[e] += jac[(size_t)9 * pt + e];
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
  jacobian_kernel<<<lbmk::cell_grid(m), 256, 0, st>>>(c.out[0], c.out[1], c.out[2], jac, c.out_dims[0],
                                                      c.out_dims[1], c.out_dims[2], inv_h);
  return cudaGetLastError();
}

cudaError_t launch_vortq(const Ctx &c, const float *jac, float *vort, float *q, int at_cells, cudaStream_t st) {
  const int m = c.out_dims[0] * c.out_dims[1] * c.out_dims[2];
  vortq_kernel<<<lbmk::cell_grid(m), 256, 0, st>>>(jac, vort, q, c.out_dims[0], c.out_dims[1], c.out_dims[2],
                                                   at_cells);
  return cudaGetLastError();
}

}  // namespace lbmh
