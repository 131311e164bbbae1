"""Pin the NumPy oracle against vectors produced by the reference itself.

The fixtures come from tack-lbm's own ``lbm.py`` kernels executed as Python
(tests/golden/make_golden.py) and from ``trt_ref.py``'s NumPy TRT step. In
float64 the oracle must reproduce them to round-off.
"""

import numpy as np
import pytest

from oracle import lbm_oracle as O
import goldens

RTOL64 = 1e-12


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / (np.abs(b) + 1e-30))) if a.size else 0.0


def test_lattice_tables():
    # lbm.py:15-18 ordering, opposite and mirror tables (lbm.py:28-35)
    assert O.CX.sum() == O.CY.sum() == O.CZ.sum() == 0
    c = np.stack([O.CX, O.CY, O.CZ], 1)
    assert (c[O.OPP] == -c).all()
    assert (c[O.MIRY] == c * [1, -1, 1]).all()
    assert (c[O.MIRZ] == c * [1, 1, -1]).all()
    assert O.W.dtype == np.float64 and np.all(O.W == O.W.astype(np.float32))
    assert abs(O.W.sum() - 1.0) < 1e-7


def test_trt_ref_numpy_and_kernel():
    z, _ = goldens.load("trt_ref")
    cfg = goldens.trt_ref_config()
    out = O.step(cfg, z["f_in"]).reshape(-1)
    # the reference kernel (float32 weights, lbm.py:48) to round-off
    assert np.max(np.abs(out - z["got"])) < 1e-15
    # trt_ref.py's NumPy step uses exact weights: within its own assertion and 1e-6 relative
    assert np.max(np.abs(out - z["ref"])) < 1e-5
    assert rel_err(out, z["ref"]) < 1e-6


@pytest.mark.parametrize("case", list(goldens.step_cases()), ids=lambda c: c["name"])
def test_step_cases(case):
    cfg = case["cfg"]
    fields = {k: v.astype(np.float64) for k, v in case["prev"].items()}
    out = O.step(cfg, case["f_in"], fields, report=case["report"]).reshape(-1)
    assert rel_err(out, case["f_out"]) < RTOL64
    assert np.array_equal(O.mask(cfg).astype(np.uint8), case["solid"])
    assert np.array_equal(O.mask(cfg, "f32").astype(np.uint8), case["solid"])
    if case["report"]:
        for k in O.FIELDS:
            np.testing.assert_allclose(fields[k], case["fields"][k], rtol=1e-11, atol=1e-15, err_msg=k)


def test_init_cases():
    z, meta = goldens.load("init_cases")
    for name, m in meta.items():
        geo = {k: m[k] for k in ("ox", "oy", "oz", "r", "hx", "hy", "hz") if k in m}
        cfg = O.Config(m["nx"], m["ny"], m["nz"], obstacle=m["obstacle"], u0=m["u0"], **geo)
        f = O.init(cfg, m["seed_amp"])
        assert rel_err(f, z[f"{name}/f"]) < RTOL64, name


def run_solver_case(m):
    """Replay make_golden.py's Solver script on the oracle (lbm.py:551-661)."""
    cfg = O.solver_config(m["nx"], m["ny"], m["nz"], collision=m["collision"], obstacle=m["obstacle"],
                          reynolds=m["reynolds"], u0=m["u0"], diameter=m["diameter"], lateral=m["lateral"])
    fields = O.new_fields(cfg.n)
    f = O.init(cfg, 0.05)
    f = O.step(cfg, f, fields, report=True).reshape(-1)
    mons = [O.monitors(cfg, fields, 1, m["diameter"])]
    cfg.omega_rot = m["rotation"]
    for _ in range(3):
        f = O.step(cfg, f).reshape(-1)
    f = O.step(cfg, f, fields, report=True).reshape(-1)
    mons.append(O.monitors(cfg, fields, 4, m["diameter"]))
    f = O.step(cfg, f).reshape(-1)
    f = O.step(cfg, f, fields, report=True).reshape(-1)
    mons.append(O.monitors(cfg, fields, 2, m["diameter"]))
    return cfg, f, fields, mons


def test_solver_cases():
    z, meta = goldens.load("solver_cases")
    for name, m in meta.items():
        cfg, f, fields, mons = run_solver_case(m)
        assert cfg.nu == m["nu"] and cfg.sponge_start == m["sponge_start"]
        assert np.array_equal(O.mask(cfg).astype(np.uint8), z[f"{name}/solid"])
        assert np.array_equal(O.mask(cfg, "f32").astype(np.uint8), z[f"{name}/solid"])
        assert rel_err(f, z[f"{name}/f"]) < 1e-11, name
        for k in O.FIELDS:
            np.testing.assert_allclose(fields[k], z[f"{name}/fields/{k}"], rtol=1e-9, atol=1e-14,
                                       err_msg=f"{name}/{k}")
        for got, want in zip(mons, m["monitors"]):
            for k, v in want.items():
                assert got[k] == pytest.approx(v, rel=1e-9, abs=1e-14), (name, k)


def weight_err(a, b):
    """max |a - b| / w_q: the error of each population relative to its lattice weight."""
    d = np.abs(np.asarray(a, np.float64).reshape(19, -1) - np.asarray(b, np.float64).reshape(19, -1))
    return float((d / O.W[:, None]).max())


def test_float32_mode_close_to_float64():
    """The reference's own arithmetic in float32 stays within 1e-6 of the
    float64 result when each population's error is scaled by its weight.
    (Pointwise relative error is not a usable yardstick: trt_ref's random
    velocities make some populations a tenth of their weight, where float32
    round-off alone reaches 2e-6.)"""
    z, _ = goldens.load("trt_ref")
    cfg = goldens.trt_ref_config()
    out32 = O.step(cfg, z["f_in"], dtype=np.float32).reshape(-1)
    assert out32.dtype == np.float32
    assert weight_err(out32, z["got"]) < 1e-6
    for case in goldens.step_cases():
        fields = {k: v.astype(np.float32) for k, v in case["prev"].items()}
        out = O.step(case["cfg"], case["f_in"], fields, report=case["report"], dtype=np.float32)
        assert weight_err(out, case["f_out"]) < 1e-6, case["name"]


@pytest.mark.parametrize("case", list(goldens.heat_cases()), ids=lambda c: c["name"])
def test_heat_step_golden(case):
    """The D3Q7 temperature block over the heat sink (lbm.py:457-492) against
    the reference kernel's own output: masks exact, populations, temperature
    and the wall heat sums to float64 round-off."""
    cfg = case["cfg"]
    assert np.array_equal(O.mask(cfg).astype(np.uint8), case["solid"])
    idx = np.arange(cfg.n)
    sink = O.sink(cfg, idx % cfg.nx, (idx // cfg.nx) % cfg.ny, idx // (cfg.nx * cfg.ny))
    assert np.array_equal(sink.astype(np.uint8), case["sink"])
    fields = {k: v.astype(np.float64) for k, v in case["prev"].items()}
    heat = {k: np.zeros(cfg.n) for k in O.HEAT_FIELDS}
    f, g = O.step_heat(cfg, case["f_in"], case["g_in"], case["t_solid"], fields, heat, report=case["report"])
    assert np.abs(f.reshape(-1) - case["f_out"]).max() < 1e-12
    assert np.abs(g.reshape(-1) - case["g_out"]).max() < 1e-12
    if case["report"]:
        assert np.abs(heat["temp"] - case["temp"]).max() < 1e-12
        assert np.abs(heat["q_solid"] - case["q_solid"]).max() < 1e-11
        for k in O.FIELDS:
            assert np.abs(fields[k] - case["fields"][k]).max() < 1e-12, k


def test_velocity_gradient_of_a_linear_field():
    """The derived-field gradient (derived.py:52-89) is exact for a linear field
    inside the grid and one-sided (still exact) at its faces; vorticity and Q of
    u = (a y, 0, 0): |curl u| = |a|, Q = 0 (pure shear)."""
    mx, my, mz = 7, 5, 4
    z, y, x = np.meshgrid(np.arange(mz), np.arange(my), np.arange(mx), indexing="ij")
    ux, uy, uz = 0.3 * x + 0.2 * y, -0.1 * z, 0.05 * x
    g = O.velocity_gradient(ux.ravel(), uy.ravel(), uz.ravel(), (mx, my, mz), 2.0)
    want = 2.0 * np.array([[0.3, 0.2, 0.0], [0.0, 0.0, -0.1], [0.05, 0.0, 0.0]])
    assert np.allclose(g, want[None], atol=1e-12)
    gs = O.velocity_gradient((0.4 * y).ravel(), 0 * x.ravel(), 0 * x.ravel(), (mx, my, mz), 1.0)
    for cells in (False, True):
        w, q = O.vorticity_q(gs, (mx, my, mz), cells)
        assert np.allclose(w, 0.4) and np.allclose(q, 0.0)


@pytest.mark.parametrize("case", list(goldens.derived_cases()), ids=lambda c: c["name"])
def test_derived_gradient_golden(case):
    """The output grid and its velocity gradient against the reference's own
    coarsen (lbm.py:516-522) and _jacobian (derived.py:52-89), run on the same
    float32 fields: identical float64 arithmetic, so equal to the bit."""
    dims = (case["nx"], case["ny"], case["nz"])
    out = [O.coarsen(case["full"][k], dims, case["stride"]) for k in ("ux", "uy", "uz")]
    for k, a in zip(("ux", "uy", "uz"), out):
        assert np.array_equal(a, case["out"][k]), k
    g = O.velocity_gradient(*out, tuple(case["out_dims"]), case["inv_h"]).reshape(-1, 9)
    assert np.array_equal(g, case["jacobian"])


@pytest.mark.parametrize("case", list(goldens.wing_cases()), ids=lambda c: c["name"])
def test_wing_step_golden(case):
    """The pitch-plunge wing step (flutter.py:61-130) against the reference kernel."""
    from oracle import flutter_oracle as FO
    cfg = case["cfg"]
    idx = np.arange(cfg.n)
    assert np.array_equal(FO.solid(cfg, idx % cfg.nx, (idx // cfg.nx) % cfg.ny).astype(np.uint8), case["solid"])
    fields = {k: np.zeros(cfg.n) for k in ("ux", "uy", "uz", "p", "vmag")}
    f, load = FO.step(cfg, case["f_in"], fields, report=case["report"])
    assert np.abs(f.reshape(-1) - case["f_out"]).max() < 1e-12
    assert np.allclose(load, case["load"], rtol=1e-12, atol=1e-12)
    if case["report"]:
        for k, v in case["fields"].items():
            assert np.abs(fields[k] - v).max() < 1e-12, k


def test_wing_init_golden():
    from oracle import flutter_oracle as FO
    cfg, f = goldens.wing_init_case()
    assert np.abs(FO.init(cfg) - f).max() < 1e-15


@pytest.mark.parametrize("case", list(goldens.fsi_cases()), ids=lambda c: c["name"])
def test_fsi_step_golden(case):
    """The cantilever-wing FSI step (fsi.py:81-186) against the reference kernel."""
    from oracle import fsi_oracle as FS
    c = case["cfg"]
    idx = np.arange(c.n)
    mask = FS.solid(c, idx % c.nx, (idx // c.nx) % c.ny, idx // (c.nx * c.ny))
    assert np.array_equal(mask.astype(np.uint8), case["solid"])
    fields = {k: np.zeros(c.n) for k in ("ux", "uy", "uz", "p", "vmag")}
    f, load = FS.step(c, case["f_in"], fields, report=case["report"])
    assert np.abs(f.reshape(-1) - case["f_out"]).max() < 1e-12
    assert np.abs(load.reshape(-1) - case["load"]).max() < 1e-11
    if case["report"]:
        for k, v in case["fields"].items():
            assert np.abs(fields[k] - v).max() < 1e-12, k
