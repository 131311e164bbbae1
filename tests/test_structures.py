"""The host-side structure integrators of the moving wings (CPU), against
closed forms.

* ``flutter.Section`` (flutter.py:134-167 in the reference): the typical
  section's uncoupled frequencies are omega_alpha in pitch and
  freq_ratio * omega_alpha in plunge; viscous damping decays the pitch
  amplitude as exp(-zeta omega t); the cubic pitch spring raises the
  frequency with amplitude (omega (1 + 3/8 H A^2) to first order).
* ``fsi.Modal`` (fsi_struct.py:176-196): each mass-normalised mode rings at
  its omega; the quartic torsion potential stiffens the torsion mode in the
  same way; undamped, the semi-implicit (symplectic) Euler keeps the energy
  bounded.
Frequencies are measured from upward zero crossings over many periods.
"""

import numpy as np
import pytest

import flutter
import fsi


def _frequency(x, dt=1.0):
    up = np.flatnonzero((x[:-1] < 0.0) & (x[1:] >= 0.0))
    # linear interpolation of the crossing times
    t = up + (-x[up]) / (x[up + 1] - x[up])
    return 2.0 * np.pi / (np.diff(t).mean() * dt)


def _ring(section, steps, pick):
    out = np.empty(steps)
    for i in range(steps):
        section.step(0.0, 0.0)
        out[i] = pick(section)
    return out


def test_section_uncoupled_frequencies():
    s = flutter.Section(24.0, x_alpha=0.0, omega_alpha=0.004, freq_ratio=0.4)
    s.v[1] = 1e-4
    pitch = _ring(s, 40000, lambda z: z.q[1])
    assert _frequency(pitch) == pytest.approx(0.004, rel=2e-3)
    s = flutter.Section(24.0, x_alpha=0.0, omega_alpha=0.004, freq_ratio=0.4)
    s.v[0] = 1e-3
    plunge = _ring(s, 60000, lambda z: z.q[0])
    assert _frequency(plunge) == pytest.approx(0.0016, rel=2e-3)


def test_section_damping_and_hardening():
    s = flutter.Section(24.0, x_alpha=0.0, omega_alpha=0.004, damping=0.01)
    s.v[1] = 1e-4
    pitch = _ring(s, 30000, lambda z: z.q[1])
    peaks = np.array([np.abs(pitch[i:i + 1500]).max() for i in (0, 28000)])
    want = np.exp(-0.01 * 0.004 * 28000)
    assert peaks[1] / peaks[0] == pytest.approx(want, rel=0.05)
    freqs = []
    for amp in (1e-4, 0.2):
        s = flutter.Section(24.0, x_alpha=0.0, omega_alpha=0.004, hardening=10.0)
        s.q[1] = amp
        freqs.append(_frequency(_ring(s, 40000, lambda z: z.q[1])))
    assert freqs[0] == pytest.approx(0.004, rel=2e-3)
    assert freqs[1] / freqs[0] == pytest.approx(1.0 + 3.0 / 8.0 * 10.0 * 0.2 ** 2, rel=0.03)


class _Modes:
    """Two modes: plunge-like (no tip twist) and twist (tip twist 0.5)."""

    def __init__(self):
        self.omega0 = np.array([0.002, 0.005])
        self.alpha = np.array([[0.0, 0.0], [0.0, 0.5]])
        self.h = np.array([[0.0, 1.0], [0.0, 0.0]])


def test_modal_frequencies_energy_and_hardening():
    fem = _Modes()
    m = fsi.Modal(fem, fem.omega0, damping=0.0, hardening=0.0, torsion=1)
    m.v[:] = [1e-3, 1e-3]
    hist = np.empty((50000, 2))
    energy = np.empty(50000)
    for i in range(50000):
        m.step(np.zeros(2))
        hist[i] = m.q
        energy[i] = 0.5 * (m.v ** 2).sum() + 0.5 * ((m.omega * m.q) ** 2).sum()
    assert _frequency(hist[:, 0]) == pytest.approx(0.002, rel=2e-3)
    assert _frequency(hist[:, 1]) == pytest.approx(0.005, rel=2e-3)
    assert energy.max() / energy.min() < 1.02
    # the quartic potential: torsion alone at tip twist amplitude A rings at
    # omega (1 + 3/8 H A^2) to first order
    m = fsi.Modal(fem, fem.omega0, hardening=20.0, torsion=1)
    amp = 0.15  # tip twist
    m.q[1] = amp / fem.alpha[1, -1]
    tw = np.empty(30000)
    for i in range(30000):
        m.step(np.zeros(2))
        tw[i] = m.q[1]
    assert _frequency(tw) / 0.005 == pytest.approx(1.0 + 3.0 / 8.0 * 20.0 * amp ** 2, rel=0.03)
    # a mode without tip twist never feels the potential
    m = fsi.Modal(fem, fem.omega0, hardening=20.0, torsion=1)
    m.q[0] = 5.0
    pl = np.empty(30000)
    for i in range(30000):
        m.step(np.zeros(2))
        pl[i] = m.q[0]
    assert _frequency(pl) == pytest.approx(0.002, rel=2e-3)
