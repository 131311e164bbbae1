"""The MFEM-free cantilever beam (tack-lbm_gb300/fsi_beam.py) against closed forms.

With the centre of gravity on the elastic axis (x_alpha = 0) bending and
torsion decouple: the twist modes of a clamped-free bar are
omega_k = (2k - 1) (pi / 2) sqrt(GJ / (I_alpha L^2)), and the shear-stiff
Timoshenko beam's first bending mode approaches Euler-Bernoulli's
1.8751^2 sqrt(EI / (m L^4)) from below. The reference (fsi_beam.py:29-126)
sets EI so that the uncoupled ratio of these two is ``freq_ratio``.
"""

import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tack-lbm_gb300"))

pytest.importorskip("scipy")

import fsi_beam  # noqa: E402


def _section(chord=32.0, mu=8.0, r_alpha2=0.5, freq_ratio=0.6, span=64.0):
    b = 0.5 * chord
    m = mu * np.pi * b * b
    i_alpha = m * r_alpha2 * b * b
    ei = m / i_alpha * (freq_ratio * np.pi * span / (2.0 * 1.875 ** 2)) ** 2
    return m, i_alpha, ei


def test_element_matrices_integrate_exactly():
    for order in (1, 2, 3, 4):
        k1, m1, d, z = fsi_beam.assemble(10.0, 5, order)
        ones = np.ones(z.size)
        assert np.abs(k1 @ ones).max() < 1e-12                # constants have no gradient
        assert abs(ones @ (m1 @ ones) - 10.0) < 1e-12          # integral of 1 over the span
        assert abs(z @ (m1 @ ones) - 50.0) < 1e-10             # integral of z
        assert abs(ones @ (d @ z) - 10.0) < 1e-12              # integral of 1 * dz/dz
        assert np.all(np.diff(z) > 0) and z[0] == 0.0 and abs(z[-1] - 10.0) < 1e-12


def test_uncoupled_modes_match_closed_forms():
    beam = fsi_beam.WingBeam(x_alpha=0.0, elements=64)
    m, i_alpha, ei = _section()
    twist = np.pi / 2 * np.sqrt(1.0 / (i_alpha * 64.0 ** 2))
    bend = 1.87510407 ** 2 * np.sqrt(ei / (m * 64.0 ** 4))
    w = beam.omega0
    # first bending below Euler-Bernoulli by the shear and rotary-inertia terms only
    assert 0.995 * bend < w[0] < bend
    assert abs(w[1] / twist - 1.0) < 1e-6
    # the second twist mode at 3x the first
    twists = [k for k in range(len(w)) if abs(beam.alpha[k, -1]) * 16.0 > abs(beam.h[k, -1])]
    assert abs(w[twists[1]] / (3.0 * twist) - 1.0) < 1e-5
    assert abs(w[0] / w[1] - 0.6) < 0.003


def test_orders_agree_and_shapes_are_signed():
    a = fsi_beam.WingBeam(order=2, elements=32)
    b = fsi_beam.WingBeam(order=3, elements=32)
    assert np.allclose(a.omega0[:4], b.omega0[:4], rtol=1e-3)  # shear-stiff: order 2 is 1e-4 high
    for beam in (a, b):
        for k in range(len(beam.omega0)):
            tip_h, tip_a = beam.h[k, -1], beam.alpha[k, -1]
            w_tip = tip_h - tip_a * (beam.elastic_axis - beam.ea) * beam.chord
            dom = w_tip if abs(w_tip) >= 16.0 * abs(tip_a) else tip_a
            assert dom > 0.0
        # the coupled model keeps the root clamped and the stations interpolate the nodes
        assert np.all(beam.h[:, 0] == 0.0) and np.all(beam.alpha[:, 0] == 0.0)
        h, al = beam.sections_at(beam.layer_z)
        assert np.allclose(h, beam.h) and np.allclose(al, beam.alpha)
        h, al = beam.sections_at([beam.span + 0.5])
        assert np.all(h == 0.0) and np.all(al == 0.0)


def test_surface_mesh():
    beam = fsi_beam.WingBeam(sections=5, contour=8)
    assert beam.rest.shape == (5 * 16, 3)
    assert beam.quads.min() >= 0 and beam.quads.max() < len(beam.rest)
    # rest state: the section outline at every station, chord along x
    xs = beam.rest[:16, 0]
    assert abs(xs.min() + beam.ea * beam.chord) < 1e-9 and abs(xs.max() - (1 - beam.ea) * beam.chord) < 1e-9
    q = np.zeros(len(beam.omega0))
    q[0] = 1.0
    moved = beam.deformed(q)
    assert moved.shape == beam.rest.shape and not np.allclose(moved, beam.rest)
