// lbm_naca.cuh - a float32 prefilter for the NACA 0012 section test of the
// moving wings (flutter.py:30-42, fsi.py:35-47).
//
// The section test is evaluated in float64 so that masks and wall fractions
// equal the float64 arithmetic exactly. On GB300 float64 issues far slower
// than float32, and nearly every cell is far from the outline, so the test
// first runs in float32 and only undecided points run the float64 form:
//   * |dx| or |dy| beyond 1.01 chord + 1 from the displaced elastic axis:
//     outside (every section point lies within 1.002 chord of it);
//   * xc below -1e-4 or above 1 + 1e-4: outside;
//   * 1e-4 <= xc <= 1 - 1e-4 and | |t| - half | > 1e-4 chord: decided by
//     the float32 comparison;
//   * anything else: undecided (the caller runs the float64 test).
// Error bound: inside the box |dx|, |dy| <= 1.02 chord, so the float32
// rotation and chord fraction err by a few 1e-7 chord (rounded inputs,
// cos/sin and 1/chord carry 6e-8 relative each), and the half-thickness by
// under 5e-6 chord for xc >= 1e-4 (the square root's slope there is 50): both
// 20x inside the margins.
#pragma once

namespace lbmk {

// Per layer (or per wing) float32 inputs of the prefilter.
struct NacaF {
  float xc0, yc0;     // elastic axis position (y includes the plunge)
  float ca, sa;       // cos, sin of the pitch
  float inv_chord, ea, half_scale;  // 1/chord, elastic-axis chord fraction, 0.6 chord
  float reach, margin;              // 1.01 chord + 1, 1e-4 chord
};

// +1 inside, -1 outside, 0 undecided.
__device__ __forceinline__ int naca_prefilter(const NacaF &k, float x, float y) {
  const float dx = x - k.xc0, dy = y - k.yc0;
  if (fabsf(dx) > k.reach || fabsf(dy) > k.reach) return -1;
  const float s = dx * k.ca - dy * k.sa, t = dx * k.sa + dy * k.ca;
  const float xc = s * k.inv_chord + k.ea;
  if (xc < -1e-4f || xc > 1.f + 1e-4f) return -1;
  if (xc < 1e-4f || xc > 1.f - 1e-4f) return 0;
  const float half = k.half_scale * (0.2969f * sqrtf(xc) - 0.1260f * xc - 0.3516f * xc * xc +
                                     0.2843f * xc * xc * xc - 0.1036f * xc * xc * xc * xc);
  const float gap = fabsf(t) - half;
  return gap < -k.margin ? 1 : (gap > k.margin ? -1 : 0);
}

inline NacaF make_naca_f(double chord, double x_ea, double yc, double ea, double ca, double sa) {
  NacaF k;
  k.xc0 = (float)x_ea;
  k.yc0 = (float)yc;
  k.ca = (float)ca;
  k.sa = (float)sa;
  k.inv_chord = (float)(1.0 / chord);
  k.ea = (float)ea;
  k.half_scale = (float)(0.6 * chord);
  k.reach = (float)(1.01 * chord + 1.0);
  k.margin = (float)(1e-4 * chord);
  return k;
}

}  // namespace lbmk
