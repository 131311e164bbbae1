"""The D3Q7 temperature block (lbm.py:457-492) and the heat sink on the GPU.

Against the reference's own outputs (tests/golden/heat_cases.npz) through
the kernel-level ``lbm_step`` and against the oracle over several steps of a
``Solver(heat=True, obstacle="heatsink")``. Tolerances: flow populations
|df|/w_q <= 1e-6 (as for every FP32 step); temperature populations
|dg|/w7_q <= 2e-6 (their values are O(1) temperatures times w7, float32
arithmetic); the temperature field 1e-6 and the wall sums q_solid 1e-5
absolute (up to six float32 atomic adds of O(1) temperatures per voxel, in
any order).
"""

import numpy as np
import pytest

from oracle import lbm_oracle as O
import goldens

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import lbm as G
    import lbm_native
    lbm_native.load()
    return G


def g_err(a, b):
    d = np.abs(np.asarray(a, np.float64).reshape(7, -1) - np.asarray(b, np.float64).reshape(7, -1))
    return float((d / O.W7[:, None]).max())


@pytest.mark.parametrize("case", list(goldens.heat_cases()), ids=lambda c: c["name"])
def test_heat_golden_through_kernel_entry(G, case):
    cfg = case["cfg"]
    n = cfg.n
    lat = G.D3Q19(cfg.nx, cfg.ny, cfg.nz)
    phys = G.COLLISIONS[cfg.collision](cfg.nu)
    geo = G.HeatSink(cfg.ny, *cfg.sink)
    flow = G.Flow(cfg.u0, cfg.sponge_start, cfg.sponge_strength, side=G.PeriodicY())
    arrays = {"t_solid": case["t_solid"].astype(np.float32), "q_solid": np.zeros(n, np.float32),
              "temp": np.zeros(n, np.float32)}
    heat = G.Heat(arrays, cfg.alpha, cfg.heat_nu)
    fields = {k: case["prev"][k].astype(np.float32).copy() for k in O.FIELDS}
    diag = (G.Report if case["report"] else G.Quiet)(fields)
    f_out = np.zeros(19 * n, np.float32)
    g_out = np.zeros(7 * n, np.float32)
    G.lbm_step(lat, phys, geo, flow, diag, case["f_in"], f_out, heat, case["g_in"], g_out)
    assert O.weight_err(f_out, case["f_out"]) <= 1e-6
    assert g_err(g_out, case["g_out"]) <= 2e-6
    if case["report"]:
        assert np.abs(arrays["temp"] - case["temp"]).max() <= 1e-6
        assert np.abs(arrays["q_solid"] - case["q_solid"]).max() <= 1e-5


def test_heatsink_solver_against_oracle(G):
    """Solver(heat=True, obstacle="heatsink"): masks exact, then flow, temperature,
    temperature field and wall sums over six steps against the oracle, with a
    warm sink (set_wall_temperature) heating an initially cold fluid."""
    nx, ny, nz, d = 40, 20, 16, 6.0
    s = G.Solver(nx, ny, nz, collision="les", obstacle="heatsink", reynolds=60.0, u0=0.05, diameter=d,
                 heat=True, prandtl=0.7, stride=2)
    cfg = O.Config(nx, ny, nz, collision="les", nu=s.nu, obstacle="heatsink", u0=0.05,
                   sponge_start=0.75 * nx, sponge_strength=1.0, heat=True, alpha=s.nu / 0.7,
                   heat_nu=s.nu, sink=tuple(s.geo.sink_params()))
    assert np.array_equal(s.mask(), O.mask(cfg).astype(np.uint8))
    assert set(s.output) == {"ux", "uy", "uz", "p", "vmag", "temp"}
    s.set_wall_temperature(1.0)
    t_solid = np.asarray(s.heat_fields["t_solid"].numpy, np.float64).copy()
    f = s.populations(np.float64)
    g = s.g[0].astype(np.float64)
    assert not g.any()  # the temperature populations start at zero (lbm.py:592)
    fields = {k: np.asarray(s.fields[k].numpy, np.float64).copy() for k in O.FIELDS}
    heat = {k: np.zeros(cfg.n) for k in O.HEAT_FIELDS}
    for k in range(6):
        rep = k in (2, 5)
        s.step(report=rep)
        if rep:
            heat["q_solid"][:] = 0.0
        f, g = O.step_heat(cfg, f, g, t_solid, fields, heat, report=rep)
        f, g = f.reshape(-1), g.reshape(-1)
        assert O.weight_err(s.populations(), f) <= 3e-6, f"step {k + 1}"
        assert g_err(s.g[0], g) <= 4e-6, f"step {k + 1}"
        if rep:
            s.sync()
            assert np.abs(s.heat_fields["temp"].numpy - heat["temp"]).max() <= 1e-6
            assert np.abs(s.heat_fields["q_solid"].numpy - heat["q_solid"]).max() <= 1e-5
    assert g.max() > 1e-3  # heat has entered the fluid
    s.monitors(6)
    coarse = s.output["temp"].numpy.reshape(s.out_dims[::-1])
    full = s.heat_fields["temp"].numpy.reshape(nz, ny, nx)
    assert np.array_equal(coarse, full[::2, ::2, ::2])
