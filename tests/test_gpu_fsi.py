"""The cantilever-wing FSI step (fsi.py:25-186) on the GPU: against the
reference's own outputs (tests/golden/fsi_cases.npz) through the kernel-level
``fsi_step``, and a released FSISolver (with a two-mode structural model)
against the oracle. Tolerances: populations |df|/w_q <= 2e-6 per FP32 step
(the interpolated bounce-back divides by 2 delta >= 1); masks exact; per-layer
loads to 1e-5 of the largest after one step and 1e-4 over coupled steps;
fields 2e-7."""

import numpy as np
import pytest

from oracle import fsi_oracle as FS
from oracle import lbm_oracle as O
import goldens

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", list(goldens.fsi_cases()), ids=lambda c: c["name"])
def test_fsi_golden_through_kernel_entry(case):
    import lbm
    import fsi
    c = case["cfg"]
    lat = lbm.D3Q19(c.nx, c.ny, c.nz)
    phys = lbm.COLLISIONS[c.collision](c.nu)
    geo = fsi.FlexWing(c.chord, c.x_ea, c.y_ea, c.ea, c.span, np.array(c.kin, np.float64))
    flow = lbm.Flow(c.u0, c.sponge_start, c.sponge_strength)
    fields = {k: np.zeros(c.n, np.float32) for k in ("ux", "uy", "uz", "p", "vmag")}
    diag = (lbm.Report if case["report"] else lbm.Quiet)(fields)
    f_out = np.zeros(19 * c.n, np.float32)
    fsi.fsi_step(lat, phys, geo, flow, diag, case["f_in"], f_out)
    assert O.weight_err(f_out, case["f_out"]) <= 2e-6
    load = case["load"].reshape(c.nz, 3)
    assert np.abs(geo.load - load).max() <= 1e-5 * np.abs(load).max()
    if case["report"]:
        for k, v in case["fields"].items():
            assert np.abs(fields[k] - v).max() <= 2e-7, k


class TwoModes:
    """A two-mode cantilever, mass normalised for a wing of modal mass ~1e4 (fluid
    density 1): bending h = A (z/span)^2, torsion alpha = B z/span."""

    A, B = 0.01, 0.002

    def __init__(self, span):
        self.span = span
        self.omega0 = np.array([0.004, 0.009])
        z = np.linspace(0.0, span, 9)
        self.h = self.A * np.stack([(z / span) ** 2, 0.1 * (z / span) ** 2])
        self.alpha = self.B * np.stack([0.0 * z, z / span])

    def sections_at(self, z):
        s = np.clip(np.asarray(z, float) / self.span, 0.0, None) * (np.asarray(z) < self.span)
        return self.A * np.stack([s ** 2, 0.1 * s ** 2]), self.B * np.stack([0.0 * s, s])


def test_fsi_solver_against_oracle():
    import fsi
    fem = TwoModes(5.5)
    s = fsi.FSISolver(48, 24, 8, chord=12.0, span=5.5, ea=0.4, u0=0.06, reynolds=150.0, collision="les",
                      reduced_velocity=3.0, damping=0.01, hardening=50.0, stride=2, fem=fem)
    assert s.torsion == 1
    ref = fsi.Modal(fem, s.structure.omega, damping=0.01, hardening=50.0, torsion=1)
    cfg = FS.FsiConfig(48, 24, 8, 12.0, 12.0, 12.0, 0.4, 5.5, kin=np.zeros((8, 4)), collision="les", nu=s.nu,
                       u0=0.06, sponge_start=36.0, sponge_strength=1.0)
    idx = np.arange(cfg.n)
    f = s.populations().astype(np.float64)
    assert O.weight_err(f, FS.init(cfg)) <= 1e-7
    s.release(tip_twist_rate=2e-4)
    ref.v[1] += 2e-4 / fem.alpha[1, -1]
    mh, ma = fem.sections_at(np.arange(8) + 0.5)
    for k in range(8):
        cfg.kin = np.stack([ref.q @ mh, ref.q @ ma, ref.v @ mh, ref.v @ ma], 1)
        mask = FS.solid(cfg, idx % cfg.nx, (idx // cfg.nx) % cfg.ny, idx // (cfg.nx * cfg.ny))
        assert np.array_equal(s.mask(), mask.astype(np.uint8)), f"step {k + 1}"
        s.step(report=(k == 7))
        f, load = FS.step(cfg, f)
        f = f.reshape(-1)
        load = load.copy()
        load[:, 2] *= -1.0
        ref.step(mh @ load[:, 1] + ma @ load[:, 2])
        assert O.weight_err(s.populations(), f) <= 6e-6, f"step {k + 1}"
        # loads are sums of (bounced + back - 2 w) over a layer's links: float32
        # round-off of several coupled steps cancels into them
        assert np.abs(s.layer_load - load).max() <= 1e-4 * max(1e-3, np.abs(load).max()), f"step {k + 1}"
    assert np.allclose(s.structure.q, ref.q, rtol=1e-3, atol=1e-12)
    assert abs(s._kin[4, 1]) > 0  # the outermost wing layer (z = 4..5) has twisted
    s.update_output()
    full = s.fields["ux"].numpy.reshape(8, 24, 48)
    assert np.array_equal(s.output["ux"].numpy.reshape(s.out_dims[::-1]), full[::2, ::2, ::2])
    assert np.isfinite(s.coefficients()).all()
    tip_h, tip_a = s.tip()
    assert np.isfinite([tip_h, tip_a]).all()


def test_fsi_solver_default_beam():
    """FSISolver with no fem= builds the bending-torsion beam (fsi.py:194) and
    couples it: the released wing's kinematics, masks and loads follow the
    oracle stepped with the same modal integrator."""
    import fsi
    from fsi_beam import WingBeam
    s = fsi.FSISolver(48, 24, 8, chord=12.0, span=5.5, ea=0.4, u0=0.06, reynolds=150.0, collision="les",
                      reduced_velocity=3.0, damping=0.01, hardening=50.0)
    beam = WingBeam(chord=12.0, span=5.5, ea=0.4)
    assert np.array_equal(s.fem.omega0, beam.omega0)
    k = s.torsion
    assert abs(beam.alpha[k, -1]) * 6.0 > abs(beam.h[k, -1])  # the first twist-dominated mode
    ref = fsi.Modal(beam, s.structure.omega, damping=0.01, hardening=50.0, torsion=k)
    cfg = FS.FsiConfig(48, 24, 8, 12.0, 12.0, 12.0, 0.4, 5.5, kin=np.zeros((8, 4)), collision="les", nu=s.nu,
                       u0=0.06, sponge_start=36.0, sponge_strength=1.0)
    idx = np.arange(cfg.n)
    f = s.populations().astype(np.float64)
    s.release()
    ref.v[k] += np.radians(2.0) * ref.omega[k] / beam.alpha[k, -1]
    mh, ma = beam.sections_at(np.arange(8) + 0.5)
    for step in range(6):
        cfg.kin = np.stack([ref.q @ mh, ref.q @ ma, ref.v @ mh, ref.v @ ma], 1)
        # the two structures are driven by the GPU's and the oracle's loads
        assert np.abs(s._kin - cfg.kin).max() <= 1e-3 * np.abs(cfg.kin).max() + 1e-15, f"step {step + 1}"
        mask = FS.solid(cfg, idx % cfg.nx, (idx // cfg.nx) % cfg.ny, idx // (cfg.nx * cfg.ny))
        assert np.array_equal(s.mask(), mask.astype(np.uint8)), f"step {step + 1}"
        s.step()
        f, load = FS.step(cfg, f)
        f = f.reshape(-1)
        load = load.copy()
        load[:, 2] *= -1.0
        ref.step(mh @ load[:, 1] + ma @ load[:, 2])
        assert O.weight_err(s.populations(), f) <= 6e-6, f"step {step + 1}"
        assert np.abs(s.layer_load - load).max() <= 1e-4 * max(1e-3, np.abs(load).max()), f"step {step + 1}"
    assert abs(s.tip()[1]) > 0.0
