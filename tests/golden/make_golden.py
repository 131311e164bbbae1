"""Generate the golden vectors under tests/golden/ from the reference itself.

Run where the tack-lbm sources are available, naming their directory as the
argument or in ``$TACK_LBM_REFERENCE``:

    python tests/golden/make_golden.py REFERENCE_DIR [--only derived,...]

The reference's kernels are Tack programs; ``tack_shim`` lets them execute
as plain Python loops in float64 (the populations and fields the reference
stores as float32 are given float32 values on input). The script writes:

* ``trt_ref.npz``   - ``trt_ref.py`` executed verbatim: its input, its NumPy TRT
                      step (``ref``) and the reference kernel's result (``got``).
* ``step_cases.npz``- one ``lbm_step`` per case over collision x obstacle x
                      lateral policy x report, from seeded near-equilibrium states.
* ``init_cases.npz``- ``lbm_init`` for each obstacle.
* ``solver_cases.npz`` - whole ``Solver`` runs: construction (init plus the
                      priming report step), quiet and report steps, a rotation
                      change and ``monitors()``.
* ``heat_cases.npz``- one ``lbm_step`` with the D3Q7 temperature block (``Heat``)
                      over the finned ``HeatSink``, quiet and report.
* ``wing_cases.npz``- one ``wing_step`` of the pitch-plunge NACA 0012 section
                      (``flutter.py``) per collision model, and ``wing_init``.
* ``fsi_cases.npz`` - one ``fsi_step`` of the cantilever wing (``fsi.py``: moving
                      layers, interpolated bounce-back, per-layer loads).
* ``derived_cases.npz`` - ``coarsen`` (lbm.py:516-522) and the derived fields'
                      velocity gradient ``_jacobian`` (derived.py:52-89) on seeded
                      output grids at strides 1, 2 and 3.

Nothing reads the reference at test time; only these files are used.
"""

import json
import os
import runpy
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import tack_shim  # noqa: E402

NX, NY, NZ = 12, 10, 6

GEOMETRY = {
    "cylinder": dict(ox=5.3, oy=4.7, oz=0.0, r=2.6),
    "sphere": dict(ox=5.5, oy=4.5, oz=2.5, r=2.4),
    "box": dict(ox=5.5, oy=5.0, oz=3.0, hx=1.5, hy=2.0, hz=1.2),
}

# (name, collision, obstacle, lateral, report, omega_rot)
STEP_CASES = [
    ("bgk_cylinder_periodic_report", "bgk", "cylinder", "periodic", True, 0.05),
    ("trt_cylinder_slip_report", "trt", "cylinder", "slip", True, -0.03),
    ("les_cylinder_slip_quiet", "les", "cylinder", "slip", False, 0.04),
    ("les_sphere_slip_report", "les", "sphere", "slip", True, 0.0),
    ("trt_sphere_periodic_quiet", "trt", "sphere", "periodic", False, 0.0),
    ("les_box_periodic_report", "les", "box", "periodic", True, 0.0),
    ("bgk_box_slip_quiet", "bgk", "box", "slip", False, 0.0),
]

SOLVER_CASES = [
    dict(name="les_cylinder_slip", nx=24, ny=16, nz=8, collision="les", obstacle="cylinder",
         reynolds=120.0, u0=0.07, diameter=6.0, lateral="slip", rotation=0.02),
    dict(name="trt_sphere_periodic", nx=24, ny=16, nz=8, collision="trt", obstacle="sphere",
         reynolds=300.0, u0=0.08, diameter=6.0, lateral="periodic", rotation=0.0),
    dict(name="bgk_box_periodic", nx=20, ny=14, nz=10, collision="bgk", obstacle="box",
         reynolds=80.0, u0=0.05, diameter=5.0, lateral="periodic", rotation=0.0),
]


def geometry(lbm, kind):
    g = GEOMETRY[kind]
    if kind == "cylinder":
        return lbm.Cylinder(g["ox"], g["oy"], g["r"])
    if kind == "sphere":
        return lbm.Sphere(g["ox"], g["oy"], g["oz"], g["r"])
    return lbm.Box(g["ox"], g["oy"], g["oz"], g["hx"], g["hy"], g["hz"])


def seeded_state(lbm, geo, n, rng):
    """Near-equilibrium float32 populations; solid cells at rest (f = w), as
    every reference step leaves them (lbm.py:449-456 with sigma = 1)."""
    c = np.array([lbm.CX, lbm.CY, lbm.CZ]).T
    w = np.array(lbm.W, np.float32).astype(np.float64)
    rho = 1 + 0.01 * rng.standard_normal(n)
    u = np.array([0.06, 0.0, 0.0]) + 0.02 * rng.standard_normal((n, 3))
    cu = 3.0 * (u @ c.T)
    f = w * rho[:, None] * (1 + cu + 0.5 * cu ** 2 - 1.5 * (u ** 2).sum(1)[:, None])
    f += 1e-3 * rng.standard_normal((n, 19))
    idx = np.arange(n)
    x, y, z = idx % NX, (idx // NX) % NY, idx // (NX * NY)
    solid = np.array([geo.solid(int(a), int(b), int(d)) for a, b, d in zip(x, y, z)])
    f[solid > 0] = w
    return np.ascontiguousarray(f.T.reshape(-1)).astype(np.float32), solid


def heat_stub(lbm, n):
    h = lbm.Solver.__new__(lbm.Solver)
    h.heat_enabled = False
    h.nx = NX
    h._setup_heat(n)
    return h


def make_trt_ref(ref_dir):
    lbm = tack_shim.import_reference(ref_dir)
    g = runpy.run_path(os.path.join(ref_dir, "trt_ref.py"), run_name="trt_ref")
    assert lbm is sys.modules["lbm"]
    err = float(np.abs(g["got"] - g["ref"]).max())
    print(f"trt_ref: max |kernel - numpy| = {err:.3e}")
    np.savez_compressed(os.path.join(HERE, "trt_ref.npz"),
                        f_in=g["f_in"], ref=g["ref"].T.reshape(-1), got=g["got"].T.reshape(-1),
                        dims=np.array([g["nx"], g["ny"], g["nz"]]), nu=np.array(0.002))


def make_step_cases(ref_dir):
    lbm = tack_shim.import_reference(ref_dir)
    n = NX * NY * NZ
    out, meta = {}, {}
    for k, (name, coll, obst, lateral, report, omega_rot) in enumerate(STEP_CASES):
        rng = np.random.default_rng(100 + k)
        lat = lbm.D3Q19(NX, NY, NZ)
        nu = 0.004 + 0.002 * k
        phys = lbm.COLLISIONS[coll](nu)
        geo = geometry(lbm, obst)
        omega = tack_shim.HostManagedArray(1)
        omega.numpy[0] = omega_rot
        side = {"periodic": lbm.PeriodicY, "slip": lbm.SlipY}[lateral]()
        u0, s0, strength = 0.06, 8.0, 0.7
        flow = lbm.Flow(u0, s0, strength, omega.tack, side)
        f_in, solid = seeded_state(lbm, geo, n, rng)
        fields = {key: tack_shim.HostManagedArray(n) for key in lbm.FIELDS}
        for key in ("ux", "uy", "uz", "p"):
            fields[key].numpy[:] = (0.02 * rng.standard_normal(n)).astype(np.float32)
        prev = {key: fields[key].numpy.copy() for key in lbm.FIELDS}
        diag = (lbm.Report if report else lbm.Quiet)({k_: v.tack for k_, v in fields.items()})
        h = heat_stub(lbm, n)
        a_in = lbm.tack.array(f_in)
        a_out = lbm.tack.empty((19 * n,))
        t0 = time.perf_counter()
        lbm.lbm_step(lat, phys, geo, flow, diag, a_in, a_out, h.heat, h.g[0], h.g[1])
        print(f"{name}: {time.perf_counter() - t0:.2f} s, solid cells {int(solid.sum())}")
        out[f"{name}/f_in"] = f_in
        out[f"{name}/f_out"] = np.asarray(a_out)
        out[f"{name}/solid"] = solid.astype(np.uint8)
        for key in lbm.FIELDS:
            out[f"{name}/prev/{key}"] = prev[key].astype(np.float32)
            if report:
                out[f"{name}/fields/{key}"] = np.asarray(fields[key].numpy)
        meta[name] = dict(nx=NX, ny=NY, nz=NZ, collision=coll, nu=nu, obstacle=obst, lateral=lateral,
                          report=report, omega_rot=omega_rot, u0=u0, sponge_start=s0,
                          sponge_strength=strength, **GEOMETRY[obst])
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "step_cases.npz"), **out)


def make_init_cases(ref_dir):
    lbm = tack_shim.import_reference(ref_dir)
    n = NX * NY * NZ
    out, meta = {}, {}
    for obst in GEOMETRY:
        lat = lbm.D3Q19(NX, NY, NZ)
        geo = geometry(lbm, obst)
        flow = lbm.Flow(0.07, 9.0, 1.0)
        f = lbm.tack.empty((19 * n,))
        lbm.lbm_init(lat, geo, flow, f, 0.05)
        out[f"{obst}/f"] = np.asarray(f)
        meta[obst] = dict(nx=NX, ny=NY, nz=NZ, obstacle=obst, u0=0.07, seed_amp=0.05, **GEOMETRY[obst])
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "init_cases.npz"), **out)


# (name, collision, report): one step with the D3Q7 temperature block over the
# finned heat sink, at the reference Solver's HeatSink placement (lbm.py:635-637)
HEAT_CASES = [("heat_les_report", "les", True), ("heat_trt_quiet", "trt", False),
              ("heat_bgk_report", "bgk", True)]
HNX, HNY, HNZ, HD = 20, 12, 16, 6.0


def heatsink_params(nx, ny, nz, d):
    """The HeatSink arguments Solver.set_obstacle("heatsink") passes (lbm.py:635-637)."""
    return (int(0.2 * nx), int(0.3 * nx), int(0.125 * nz), int(0.75 * nz), round(d / 2), int(0.45 * ny),
            round(d / 3), round(d))


def make_heat_cases(ref_dir):
    lbm = tack_shim.import_reference(ref_dir)
    n = HNX * HNY * HNZ
    sink = heatsink_params(HNX, HNY, HNZ, HD)
    out, meta = {}, {}
    for k, (name, coll, report) in enumerate(HEAT_CASES):
        rng = np.random.default_rng(300 + k)
        lat = lbm.D3Q19(HNX, HNY, HNZ)
        nu = 0.01 + 0.003 * k
        phys = lbm.COLLISIONS[coll](nu)
        geo = lbm.HeatSink(HNY, *sink)
        omega = tack_shim.HostManagedArray(1)
        u0, s0, strength = 0.05, 15.0, 0.8
        flow = lbm.Flow(u0, s0, strength, omega.tack, lbm.PeriodicY())
        idx = np.arange(n)
        x, y, z = idx % HNX, (idx // HNX) % HNY, idx // (HNX * HNY)
        solid = np.array([geo.solid(int(a), int(b), int(c)) for a, b, c in zip(x, y, z)])
        hot = np.array([geo.sink(int(a), int(b), int(c)) for a, b, c in zip(x, y, z)])
        cvec = np.array([lbm.CX, lbm.CY, lbm.CZ]).T
        w = np.array(lbm.W, np.float32).astype(np.float64)
        rho = 1 + 0.01 * rng.standard_normal(n)
        u = np.array([u0, 0.0, 0.0]) + 0.02 * rng.standard_normal((n, 3))
        cu = 3.0 * (u @ cvec.T)
        f = w * rho[:, None] * (1 + cu + 0.5 * cu ** 2 - 1.5 * (u ** 2).sum(1)[:, None])
        f += 1e-3 * rng.standard_normal((n, 19))
        f[solid > 0] = w
        f_in = np.ascontiguousarray(f.T.reshape(-1)).astype(np.float32)
        # temperature populations near w7 T with T in [0, 1]; zero in solid cells
        w7 = np.array(lbm.W7, np.float32).astype(np.float64)
        temp = rng.uniform(0.0, 1.0, n)
        g = w7 * temp[:, None] + 0.01 * rng.standard_normal((n, 7))
        g[solid > 0] = 0.0
        g_in = np.ascontiguousarray(g.T.reshape(-1)).astype(np.float32)
        t_solid = np.where(hot > 0, rng.uniform(0.5, 1.5, n), 0.0).astype(np.float32)
        fields = {key: tack_shim.HostManagedArray(n) for key in lbm.FIELDS}
        prev = {key: fields[key].numpy.copy() for key in lbm.FIELDS}
        diag = (lbm.Report if report else lbm.Quiet)({k_: v.tack for k_, v in fields.items()})
        st = lbm.Solver.__new__(lbm.Solver)
        st.heat_enabled, st.nu, st.prandtl, st.nx = True, nu, 0.7, HNX
        st._setup_heat(n)
        st.heat_fields["t_solid"].numpy[:] = t_solid
        st.heat_fields["q_solid"].numpy[:] = 0.0
        a_in = lbm.tack.array(f_in)
        a_out = lbm.tack.empty((19 * n,))
        g_a = lbm.tack.array(g_in)
        g_b = lbm.tack.zeros((7 * n,))
        t0 = time.perf_counter()
        lbm.lbm_step(lat, phys, geo, flow, diag, a_in, a_out, st.heat, g_a, g_b)
        print(f"{name}: {time.perf_counter() - t0:.2f} s, solid {int(solid.sum())}, sink {int(hot.sum())}")
        out[f"{name}/f_in"] = f_in
        out[f"{name}/g_in"] = g_in
        out[f"{name}/t_solid"] = t_solid
        out[f"{name}/f_out"] = np.asarray(a_out)
        out[f"{name}/g_out"] = np.asarray(g_b)
        out[f"{name}/solid"] = solid.astype(np.uint8)
        out[f"{name}/sink"] = hot.astype(np.uint8)
        if report:
            out[f"{name}/temp"] = np.asarray(st.heat_fields["temp"].numpy)
            out[f"{name}/q_solid"] = np.asarray(st.heat_fields["q_solid"].numpy)
            for key in lbm.FIELDS:
                out[f"{name}/fields/{key}"] = np.asarray(fields[key].numpy)
        for key in lbm.FIELDS:
            out[f"{name}/prev/{key}"] = prev[key].astype(np.float32)
        meta[name] = dict(nx=HNX, ny=HNY, nz=HNZ, collision=coll, nu=nu, obstacle="heatsink",
                          lateral="periodic", report=report, u0=u0, sponge_start=s0,
                          sponge_strength=strength, sink=list(sink), heat=True, alpha=nu / 0.7,
                          heat_nu=nu)
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "heat_cases.npz"), **out)


# (name, collision, report, state h, alpha, dh/dt, dalpha/dt): one wing_step of
# the pitch-plunge NACA 0012 section (flutter.py:20-130)
WING_CASES = [("wing_les_report", "les", True, (0.7, 0.12, 0.003, 0.0015)),
              ("wing_trt_quiet", "trt", False, (-1.2, -0.2, -0.002, 0.001)),
              ("wing_bgk_report", "bgk", True, (0.0, 0.05, 0.0, -0.002))]
WNX, WNY, WNZ, WCHORD, WEA = 48, 24, 2, 16.0, 0.4


def import_flutter(ref_dir):
    lbm = tack_shim.import_reference(ref_dir)
    sys.modules.pop("flutter", None)
    import flutter  # noqa: E402  (the reference module, on the shim)
    import math
    flutter.sqrt, flutter.sin, flutter.cos = math.sqrt, math.sin, math.cos
    return lbm, flutter


def make_wing_cases(ref_dir):
    lbm, flutter = import_flutter(ref_dir)
    n = WNX * WNY * WNZ
    out, meta = {}, {}
    for k, (name, coll, report, state) in enumerate(WING_CASES):
        rng = np.random.default_rng(500 + k)
        lat = lbm.D3Q19(WNX, WNY, WNZ)
        nu = 0.01 + 0.004 * k
        phys = lbm.COLLISIONS[coll](nu)
        st = tack_shim.HostManagedArray(4)
        st.numpy[:] = state
        load = tack_shim.HostManagedArray(3)
        geo = flutter.Wing(WCHORD, 0.25 * WNX, 0.5 * WNY, WEA, st.tack, load.tack)
        u0, s0, strength = 0.06, 36.0, 0.9
        flow = lbm.Flow(u0, s0, strength)
        idx = np.arange(n)
        x, y, z = idx % WNX, (idx // WNX) % WNY, idx // (WNX * WNY)
        solid = np.array([geo.solid(int(a), int(b), int(c)) for a, b, c in zip(x, y, z)])
        cvec = np.array([lbm.CX, lbm.CY, lbm.CZ]).T
        w = np.array(lbm.W, np.float32).astype(np.float64)
        rho = 1 + 0.01 * rng.standard_normal(n)
        u = np.array([u0, 0.0, 0.0]) + 0.02 * rng.standard_normal((n, 3))
        cu = 3.0 * (u @ cvec.T)
        f = w * rho[:, None] * (1 + cu + 0.5 * cu ** 2 - 1.5 * (u ** 2).sum(1)[:, None])
        f += 1e-3 * rng.standard_normal((n, 19))
        f_in = np.ascontiguousarray(f.T.reshape(-1)).astype(np.float32)
        fields = {key: tack_shim.HostManagedArray(n) for key in lbm.FIELDS}
        diag = (lbm.Report if report else lbm.Quiet)({k_: v.tack for k_, v in fields.items()})
        a_in = lbm.tack.array(f_in)
        a_out = lbm.tack.empty((19 * n,))
        t0 = time.perf_counter()
        flutter.wing_step(lat, phys, geo, flow, diag, a_in, a_out)
        print(f"{name}: {time.perf_counter() - t0:.2f} s, solid {int(solid.sum())}, load {load.numpy}")
        out[f"{name}/f_in"] = f_in
        out[f"{name}/f_out"] = np.asarray(a_out)
        out[f"{name}/solid"] = solid.astype(np.uint8)
        out[f"{name}/load"] = np.asarray(load.numpy)
        if report:
            for key in ("ux", "uy", "uz", "p", "vmag"):
                out[f"{name}/fields/{key}"] = np.asarray(fields[key].numpy)
        meta[name] = dict(nx=WNX, ny=WNY, nz=WNZ, collision=coll, nu=nu, report=report, u0=u0,
                          sponge_start=s0, sponge_strength=strength, chord=WCHORD, x_ea=0.25 * WNX,
                          y_ea=0.5 * WNY, ea=WEA, state=list(state))
    # wing_init at a displaced state
    lat = lbm.D3Q19(WNX, WNY, WNZ)
    st = tack_shim.HostManagedArray(4)
    st.numpy[:] = (0.5, -0.1, 0.0, 0.0)
    geo = flutter.Wing(WCHORD, 0.25 * WNX, 0.5 * WNY, WEA, st.tack, tack_shim.HostManagedArray(3).tack)
    f0 = lbm.tack.empty((19 * n,))
    flutter.wing_init(lat, geo, lbm.Flow(0.06, 36.0, 0.9), f0)
    out["init/f"] = np.asarray(f0)
    meta["init"] = dict(nx=WNX, ny=WNY, nz=WNZ, u0=0.06, chord=WCHORD, x_ea=0.25 * WNX, y_ea=0.5 * WNY,
                        ea=WEA, state=[0.5, -0.1, 0.0, 0.0])
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "wing_cases.npz"), **out)


# (name, collision, report): one fsi_step of the cantilever wing (fsi.py:25-186)
# with a different plunge/pitch and rates in every layer
FSI_CASES = [("fsi_les_report", "les", True), ("fsi_trt_quiet", "trt", False), ("fsi_bgk_report", "bgk", True)]
FNX, FNY, FNZ, FCHORD, FSPAN, FEA = 36, 20, 8, 12.0, 5.5, 0.4


def import_fsi(ref_dir):
    """The reference fsi module on the shim. Its structural modules import MFEM at
    module level; the kernels do not use it, so empty stand-in modules let the
    file import (nothing of MFEM is called)."""
    import math
    import types
    lbm = tack_shim.import_reference(ref_dir)

    class _Stand(types.ModuleType):
        def __getattr__(self, name):  # classes the structural modules derive from at import
            return type(name, (), {})

    mf = _Stand("mfem")
    mf.ser = _Stand("mfem.ser")
    sys.modules["mfem"], sys.modules["mfem.ser"] = mf, mf.ser
    for name in ("fsi", "fsi_beam", "fsi_struct"):
        sys.modules.pop(name, None)
    import fsi  # noqa: E402  (the reference module, on the shim)
    fsi.sqrt, fsi.sin, fsi.cos = math.sqrt, math.sin, math.cos
    return lbm, fsi


def fsi_kinematics(rng):
    z = np.arange(FNZ) + 0.5
    kin = np.zeros((FNZ, 4))
    kin[:, 0] = 0.8 * (z / FSPAN) ** 2 + 0.05 * rng.standard_normal(FNZ)
    kin[:, 1] = 0.15 * (z / FSPAN) + 0.02 * rng.standard_normal(FNZ)
    kin[:, 2] = 0.004 * (z / FSPAN) ** 2
    kin[:, 3] = -0.002 * (z / FSPAN)
    return kin


def make_fsi_cases(ref_dir):
    lbm, fsi = import_fsi(ref_dir)
    n = FNX * FNY * FNZ
    out, meta = {}, {}
    reflect = fsi._reflect_z()
    for k, (name, coll, report) in enumerate(FSI_CASES):
        rng = np.random.default_rng(700 + k)
        lat = lbm.D3Q19(FNX, FNY, FNZ)
        nu = 0.008 + 0.003 * k
        phys = lbm.COLLISIONS[coll](nu)
        kin_a = tack_shim.HostManagedArray(4 * FNZ)
        kin = fsi_kinematics(rng)
        kin_a.numpy[:] = kin.reshape(-1)
        load = tack_shim.HostManagedArray(3 * FNZ)
        geo = fsi.FlexWing(FCHORD, 0.25 * FNX, 0.5 * FNY, FEA, FSPAN, kin_a.tack, load.tack, reflect)
        u0, s0, strength = 0.06, 27.0, 0.9
        flow = lbm.Flow(u0, s0, strength)
        cvec = np.array([lbm.CX, lbm.CY, lbm.CZ]).T
        w = np.array(lbm.W, np.float32).astype(np.float64)
        rho = 1 + 0.01 * rng.standard_normal(n)
        u = np.array([u0, 0.0, 0.0]) + 0.02 * rng.standard_normal((n, 3))
        cu = 3.0 * (u @ cvec.T)
        f = w * rho[:, None] * (1 + cu + 0.5 * cu ** 2 - 1.5 * (u ** 2).sum(1)[:, None])
        f += 1e-3 * rng.standard_normal((n, 19))
        f_in = np.ascontiguousarray(f.T.reshape(-1)).astype(np.float32)
        idx = np.arange(n)
        x, y, z = idx % FNX, (idx // FNX) % FNY, idx // (FNX * FNY)
        solid = np.array([geo.solid(int(a), int(b), int(c)) for a, b, c in zip(x, y, z)])
        fields = {key: tack_shim.HostManagedArray(n) for key in lbm.FIELDS}
        diag = (lbm.Report if report else lbm.Quiet)({k_: v.tack for k_, v in fields.items()})
        a_in = lbm.tack.array(f_in)
        a_out = lbm.tack.empty((19 * n,))
        t0 = time.perf_counter()
        fsi.fsi_step(lat, phys, geo, flow, diag, a_in, a_out)
        print(f"{name}: {time.perf_counter() - t0:.2f} s, solid {int(solid.sum())}")
        out[f"{name}/f_in"] = f_in
        out[f"{name}/f_out"] = np.asarray(a_out)
        out[f"{name}/solid"] = solid.astype(np.uint8)
        out[f"{name}/kin"] = kin
        out[f"{name}/load"] = np.asarray(load.numpy)
        if report:
            for key in ("ux", "uy", "uz", "p", "vmag"):
                out[f"{name}/fields/{key}"] = np.asarray(fields[key].numpy)
        meta[name] = dict(nx=FNX, ny=FNY, nz=FNZ, collision=coll, nu=nu, report=report, u0=u0,
                          sponge_start=s0, sponge_strength=strength, chord=FCHORD, x_ea=0.25 * FNX,
                          y_ea=0.5 * FNY, ea=FEA, span=FSPAN)
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "fsi_cases.npz"), **out)


def make_solver_cases(ref_dir):
    lbm = tack_shim.import_reference(ref_dir)
    out, meta = {}, {}
    for case in SOLVER_CASES:
        c = dict(case)
        name, rotation = c.pop("name"), c.pop("rotation")
        t0 = time.perf_counter()
        s = lbm.Solver(**c)
        mon0 = s.monitors(1)
        s.set_actuation(rotation)
        for _ in range(3):
            s.step()
        s.step(report=True)
        mon1 = s.monitors(4)
        s.step()
        s.step(report=True)
        mon2 = s.monitors(2)
        print(f"solver {name}: {time.perf_counter() - t0:.1f} s, steps {s.step_count}, "
              f"drag {mon2['drag']:.5f} lift {mon2['lift']:.5f}")
        out[f"{name}/f"] = np.asarray(s.f[0])
        out[f"{name}/solid"] = np.array([s.geo.solid(i % s.nx, (i // s.nx) % s.ny, i // (s.nx * s.ny))
                                         for i in range(s.lat.n)], np.uint8)
        for key in lbm.FIELDS:
            out[f"{name}/fields/{key}"] = np.asarray(s.fields[key].numpy)
        meta[name] = dict(case, monitors=[mon0, mon1, mon2], step_count=s.step_count,
                          nu=s.nu, sponge_start=s.flow.sponge_start)
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "solver_cases.npz"), **out)


# (name, full lattice (nx, ny, nz), output stride, diameter): derived-field cases.
# Odd sizes make the coarsened grid ceil(n / stride); nz = 1 and stride 3 over
# nz = 4 give one- and two-point axes (a zero and a one-sided z derivative).
DERIVED_CASES = [
    ("stride1", (20, 12, 7), 1, 8.0),
    ("stride2_odd", (21, 13, 7), 2, 8.0),
    ("flat_z", (16, 10, 1), 1, 6.0),
    ("stride3_thin", (17, 9, 4), 3, 12.0),
]


def import_derived(ref_dir):
    """The reference derived module on the shim. It imports tack.dataset and the
    tack-expr compiler at module level; ``_jacobian`` and ``coarsen`` use
    neither, so empty stand-in modules let the file import."""
    import types
    lbm = tack_shim.import_reference(ref_dir)
    tack = sys.modules["tack"]
    td = types.ModuleType("tack.dataset")
    tack.dataset = td
    sys.modules["tack.dataset"] = td
    sys.modules["tack_expr"] = types.ModuleType("tack_expr")
    sys.modules.pop("derived", None)
    import derived  # noqa: E402  (the reference module, on the shim)
    return lbm, derived


def derived_fields(nx, ny, nz, rng):
    """Seeded float32 velocity fields: a developing-wake-like shear flow plus noise."""
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ux = 0.08 * np.tanh((y - ny / 2) / 3.0) * np.cos(2 * np.pi * x / nx) + 0.05
    uy = 0.03 * np.sin(2 * np.pi * x / nx + 0.4 * z) * np.exp(-((y - ny / 2) / 4.0) ** 2)
    uz = 0.01 * np.cos(2 * np.pi * (x + 2 * y) / nx) * np.sin(np.pi * (z + 0.5) / max(nz, 1))
    out = []
    for a in (ux, uy, uz):
        a = a + 2e-3 * rng.standard_normal(a.shape)
        out.append(a.astype(np.float32).reshape(-1))
    return out


def make_derived_cases(ref_dir):
    """The reference's own coarsen (lbm.py:516-522) and velocity gradient
    ``_jacobian`` (derived.py:52-89, gradient="lattice") on seeded fields, with
    inv_h = 1 / h, h = stride / diameter (derived.py:101-103)."""
    lbm, derived = import_derived(ref_dir)
    rng = np.random.default_rng(20241204)
    out, meta = {}, {}
    for name, (nx, ny, nz), stride, diameter in DERIVED_CASES:
        t0 = time.time()
        lat = lbm.D3Q19(nx, ny, nz)
        full = derived_fields(nx, ny, nz, rng)
        mx, my, mz = ((d + stride - 1) // stride for d in (nx, ny, nz))
        m = mx * my * mz
        coarse = []
        for a in full:
            dst = np.zeros(m)
            lbm.coarsen(lat, stride, a.astype(np.float64), dst, mx, my, mz)
            coarse.append(dst)
        inv_h = 1.0 / (stride / diameter)
        jac = np.zeros((m, 9))
        derived._jacobian(coarse[0], coarse[1], coarse[2], jac, mx, my, mz, inv_h)
        for key, a in zip(("ux", "uy", "uz"), full):
            out[f"{name}/{key}"] = a
        for key, a in zip(("ux", "uy", "uz"), coarse):
            out[f"{name}/out_{key}"] = a.astype(np.float32)
        out[f"{name}/jacobian"] = jac
        meta[name] = dict(nx=nx, ny=ny, nz=nz, stride=stride, diameter=diameter, out_dims=[mx, my, mz],
                          inv_h=inv_h)
        print(f"derived {name}: {time.time() - t0:.1f} s")
    out["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "derived_cases.npz"), **out)


MAKERS = {"trt_ref": make_trt_ref, "step": make_step_cases, "init": make_init_cases,
          "solver": make_solver_cases, "heat": make_heat_cases, "wing": make_wing_cases,
          "fsi": make_fsi_cases, "derived": make_derived_cases}


def main():
    import argparse
    ap = argparse.ArgumentParser(description="Write tests/golden/*.npz from the tack-lbm sources.")
    ap.add_argument("reference_dir", nargs="?", default=os.environ.get("TACK_LBM_REFERENCE"),
                    help="directory holding tack-lbm's lbm.py, trt_ref.py, flutter.py, fsi.py and "
                         "derived.py (default: $TACK_LBM_REFERENCE)")
    ap.add_argument("--only", default=",".join(MAKERS),
                    help=f"comma list of the fixture sets to write (default all: {','.join(MAKERS)})")
    args = ap.parse_args()
    if not args.reference_dir:
        ap.error("give the tack-lbm source directory as an argument or in $TACK_LBM_REFERENCE")
    if not os.path.isfile(os.path.join(args.reference_dir, "lbm.py")):
        ap.error(f"{args.reference_dir} holds no lbm.py")
    names = [s.strip() for s in args.only.split(",") if s.strip()]
    bad = [s for s in names if s not in MAKERS]
    if bad:
        ap.error(f"unknown fixture sets {bad}")
    for name in names:
        MAKERS[name](args.reference_dir)


if __name__ == "__main__":
    main()
