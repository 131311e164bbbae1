"""The pitch-plunge wing step (flutter.py:20-130) on the GPU: against the
reference's own outputs (tests/golden/wing_cases.npz) through the kernel-level
``wing_step``, and a released FlutterSolver against the oracle with the
structure integrated alongside. Tolerances: populations |df|/w_q <= 1e-6 (an
FP32 step); masks exact; the summed force and moment to 2e-6 of their size
(float32 block sums added in float64)."""

import numpy as np
import pytest

from oracle import flutter_oracle as FO
from oracle import lbm_oracle as O
import goldens

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", list(goldens.wing_cases()), ids=lambda c: c["name"])
def test_wing_golden_through_kernel_entry(case):
    import lbm
    import flutter
    c = case["cfg"]
    lat = lbm.D3Q19(c.nx, c.ny, c.nz)
    phys = lbm.COLLISIONS[c.collision](c.nu)
    geo = flutter.Wing(c.chord, c.x_ea, c.y_ea, c.ea, state=np.array(c.state, np.float64))
    flow = lbm.Flow(c.u0, c.sponge_start, c.sponge_strength)
    fields = {k: np.zeros(c.n, np.float32) for k in ("ux", "uy", "uz", "p", "vmag")}
    diag = (lbm.Report if case["report"] else lbm.Quiet)(fields)
    f_out = np.zeros(19 * c.n, np.float32)
    flutter.wing_step(lat, phys, geo, flow, diag, case["f_in"], f_out)
    assert O.weight_err(f_out, case["f_out"]) <= 1e-6
    load = case["load"]
    assert np.abs(geo.load - load).max() <= 2e-6 * np.abs(load).max()
    if case["report"]:
        for k, v in case["fields"].items():
            assert np.abs(fields[k] - v).max() <= 2e-7, k


def test_wing_init_golden():
    import lbm
    import flutter
    c, f = goldens.wing_init_case()
    lat = lbm.D3Q19(c.nx, c.ny, c.nz)
    geo = flutter.Wing(c.chord, c.x_ea, c.y_ea, c.ea, state=np.array(c.state, np.float64))
    out = np.zeros(19 * c.n, np.float32)
    flutter.wing_init(lat, geo, lbm.Flow(c.u0, 36.0, 0.9), out)
    assert O.weight_err(out, f) <= 1e-7


def test_flutter_solver_against_oracle():
    """A released wing: 12 coupled steps (fluid on the GPU, structure on the host)
    against the oracle step driving the same Section arithmetic."""
    import flutter
    s = flutter.FlutterSolver(96, 48, 2, chord=24.0, ea=0.4, u0=0.08, reynolds=300.0, collision="les",
                              stride=2, mu=5.0, omega_alpha=0.01)
    cfg = FO.WingConfig(96, 48, 2, 24.0, 0.25 * 96, 0.5 * 48, 0.4, collision="les", nu=s.nu, u0=0.08,
                        sponge_start=0.75 * 96, sponge_strength=1.0)
    f = s.populations().astype(np.float64)
    ref = flutter.Section(12.0, mu=5.0, omega_alpha=0.01)
    s.release(alpha_rate=0.002)
    ref.v[1] += 0.002
    for k in range(12):
        cfg.state = (ref.q[0], ref.q[1], ref.v[0], ref.v[1])
        idx = np.arange(cfg.n)
        assert np.array_equal(s.mask(), FO.solid(cfg, idx % cfg.nx, (idx // cfg.nx) % cfg.ny).astype(np.uint8))
        s.step(report=(k == 11))
        f, (fx, fy, mz) = FO.step(cfg, f)
        f = f.reshape(-1)
        ref.step(fy / cfg.nz, -mz / cfg.nz)
        assert O.weight_err(s.populations(), f) <= 5e-6, f"step {k + 1}"
        assert abs(s.lift - fy / cfg.nz) <= 1e-5 * max(1.0, abs(fy / cfg.nz)), f"step {k + 1}"
        assert np.allclose(s.section.q, ref.q, rtol=1e-4, atol=1e-9)
    assert abs(s.section.q[1]) > 0  # the wing moved
    s.update_output()
    full = s.fields["ux"].numpy.reshape(2, 48, 96)
    assert np.array_equal(s.output["ux"].numpy.reshape(s.out_dims[::-1]), full[::2, ::2, ::2])
    cd, cl, cm = s.coefficients()
    assert np.isfinite([cd, cl, cm]).all()
