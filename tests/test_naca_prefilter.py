"""The float32 prefilter of the wing section test (tack-lbm_gb300/csrc/lbm_naca.cuh)
never decides against the float64 test (flutter.py:30-42, fsi.py:35-47).

The prefilter's arithmetic is restated here in float32 NumPy, once as written
and once with every product-sum contracted to one rounding (as a fused
multiply-add on the GPU may do), and compared with the oracle's float64 test
on points spread over the wing, on points within a thousandth of a cell of
its outline and on the exact link midpoints the wall bisection visits. A
decided point must agree; undecided points go to the float64 test, and their
share must stay small for the filter to pay."""

import numpy as np

from oracle.flutter_oracle import THICK

F = np.float32


def prefilter(x, y, chord, x_ea, yc, ea, a, fused):
    """+1 inside, -1 outside, 0 undecided: the device code in float32."""
    ca, sa = F(np.cos(a)), F(np.sin(a))
    xc0, yc0 = F(x_ea), F(yc)
    inv, eaf, hs = F(1.0 / chord), F(ea), F(0.6 * chord)
    reach, margin = F(1.01 * chord + 1.0), F(1e-4 * chord)
    dx, dy = F(x) - xc0, F(y) - yc0
    if fused:  # one rounding per product-sum
        s = (dx.astype(np.float64) * ca - dy.astype(np.float64) * sa).astype(F)
        t = (dx.astype(np.float64) * sa + dy.astype(np.float64) * ca).astype(F)
        xc = (s.astype(np.float64) * inv + eaf).astype(F)
    else:
        s = dx * ca - dy * sa
        t = dx * sa + dy * ca
        xc = s * inv + eaf
    c = np.clip(xc, F(0), F(1))
    half = hs * (F(THICK[0]) * np.sqrt(c) + F(THICK[1]) * c + F(THICK[2]) * c * c + F(THICK[3]) * c * c * c
                 + F(THICK[4]) * c * c * c * c)
    gap = np.abs(t) - half
    r = np.where(gap < -margin, 1, np.where(gap > margin, -1, 0))
    r = np.where((xc < F(1e-4)) | (xc > F(1) - F(1e-4)), 0, r)
    r = np.where((xc < F(-1e-4)) | (xc > F(1) + F(1e-4)), -1, r)
    r = np.where((np.abs(dx) > reach) | (np.abs(dy) > reach), -1, r)
    return r


def section64(x, y, chord, x_ea, yc, ea, a):
    dx, dy = np.asarray(x, np.float64) - x_ea, np.asarray(y, np.float64) - yc
    s = dx * np.cos(a) - dy * np.sin(a)
    t = dx * np.sin(a) + dy * np.cos(a)
    xc = s / chord + ea
    c = np.clip(xc, 0.0, 1.0)
    half = 0.6 * chord * (THICK[0] * np.sqrt(c) + THICK[1] * c + THICK[2] * c ** 2 + THICK[3] * c ** 3
                          + THICK[4] * c ** 4)
    return (xc >= 0.0) & (xc <= 1.0) & (np.abs(t) < half)


def test_prefilter_agrees_with_float64():
    rng = np.random.default_rng(7)
    undecided, total = 0, 0
    for trial in range(24):
        chord = float(rng.choice([12.0, 32.0, 48.0, 96.0]))
        x_ea, ea = float(rng.uniform(30, 400)), float(rng.uniform(0.25, 0.5))
        yc = float(rng.uniform(30, 300) + rng.normal(0, 0.1 * chord))
        a = float(rng.normal(0, 0.3))
        # lattice points around the wing, and link points at k/64 offsets
        gx, gy = np.meshgrid(np.arange(int(x_ea - 1.2 * chord), int(x_ea + 1.2 * chord) + 1),
                             np.arange(int(yc - 1.2 * chord), int(yc + 1.2 * chord) + 1))
        gx, gy = gx.ravel().astype(np.float64), gy.ravel().astype(np.float64)
        k = rng.integers(0, 64, gx.size) / 64.0
        d = rng.integers(-1, 2, (2, gx.size))
        lx, ly = gx - k * d[0], gy - k * d[1]
        # points within 1e-3 of the outline (outside and inside)
        xs = rng.uniform(0, 1, 20000)
        half = 0.6 * chord * (THICK[0] * np.sqrt(xs) + THICK[1] * xs + THICK[2] * xs ** 2 + THICK[3] * xs ** 3
                              + THICK[4] * xs ** 4)
        tt = np.sign(rng.uniform(-1, 1, xs.size)) * (half + rng.uniform(-1e-3, 1e-3, xs.size))
        ss = (xs - ea) * chord
        ox = x_ea + ss * np.cos(a) + tt * np.sin(a)
        oy = yc - ss * np.sin(a) + tt * np.cos(a)
        for x, y in ((gx, gy), (lx, ly), (ox, oy)):
            # the outline points are not float32-exact: test the float32 point itself
            x32, y32 = F(x).astype(np.float64), F(y).astype(np.float64)
            exact = section64(x32, y32, chord, x_ea, yc, ea, a)
            for fused in (False, True):
                r = prefilter(x32, y32, chord, x_ea, yc, ea, a, fused)
                decided = r != 0
                assert np.array_equal((r[decided] > 0), exact[decided]), (trial, fused)
                if x is gx:
                    undecided += int((~decided).sum())
                    total += x.size
    assert undecided < 0.01 * total
