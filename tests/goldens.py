"""Loaders for the golden vectors in tests/golden/ (made by make_golden.py)."""

import json
import os

import numpy as np

from oracle import lbm_oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"])) if "meta" in z.files else None
    return z, meta


def trt_ref_config():
    """trt_ref.py:27-29: TRT(0.002), Cylinder(-100, -100, 0), Flow(0, 1e9, 0)."""
    z, _ = load("trt_ref")
    nx, ny, nz = (int(v) for v in z["dims"])
    return O.Config(nx, ny, nz, collision="trt", nu=float(z["nu"]), obstacle="cylinder",
                    ox=-100.0, oy=-100.0, r=0.0, u0=0.0, sponge_start=1e9, sponge_strength=0.0)


def step_case_config(m):
    keys = ("collision", "nu", "obstacle", "lateral", "omega_rot", "u0", "sponge_start",
            "sponge_strength", "ox", "oy", "oz", "r", "hx", "hy", "hz")
    return O.Config(m["nx"], m["ny"], m["nz"], **{k: m[k] for k in keys if k in m})


def step_cases():
    z, meta = load("step_cases")
    for name, m in meta.items():
        case = {"name": name, "cfg": step_case_config(m), "report": m["report"],
                "f_in": z[f"{name}/f_in"], "f_out": z[f"{name}/f_out"], "solid": z[f"{name}/solid"],
                "prev": {k: z[f"{name}/prev/{k}"] for k in O.FIELDS}}
        if m["report"]:
            case["fields"] = {k: z[f"{name}/fields/{k}"] for k in O.FIELDS}
        yield case


def heat_case_config(m):
    keys = ("collision", "nu", "obstacle", "lateral", "u0", "sponge_start", "sponge_strength",
            "alpha", "heat_nu")
    return O.Config(m["nx"], m["ny"], m["nz"], sink=tuple(m["sink"]), heat=True,
                    **{k: m[k] for k in keys})


def heat_cases():
    z, meta = load("heat_cases")
    for name, m in meta.items():
        case = {"name": name, "cfg": heat_case_config(m), "report": m["report"],
                **{k: z[f"{name}/{k}"] for k in ("f_in", "g_in", "t_solid", "f_out", "g_out", "solid", "sink")},
                "prev": {k: z[f"{name}/prev/{k}"] for k in O.FIELDS}}
        if m["report"]:
            case["temp"] = z[f"{name}/temp"]
            case["q_solid"] = z[f"{name}/q_solid"]
            case["fields"] = {k: z[f"{name}/fields/{k}"] for k in O.FIELDS}
        yield case


def wing_cases():
    from oracle import flutter_oracle as FO
    z, meta = load("wing_cases")
    for name, m in meta.items():
        if name == "init":
            continue
        keys = ("collision", "nu", "u0", "sponge_start", "sponge_strength", "chord", "x_ea", "y_ea", "ea")
        cfg = FO.WingConfig(m["nx"], m["ny"], m["nz"], state=tuple(m["state"]), **{k: m[k] for k in keys})
        case = {"name": name, "cfg": cfg, "report": m["report"], "f_in": z[f"{name}/f_in"],
                "f_out": z[f"{name}/f_out"], "solid": z[f"{name}/solid"], "load": z[f"{name}/load"]}
        if m["report"]:
            case["fields"] = {k: z[f"{name}/fields/{k}"] for k in ("ux", "uy", "uz", "p", "vmag")}
        yield case


def wing_init_case():
    from oracle import flutter_oracle as FO
    z, meta = load("wing_cases")
    m = meta["init"]
    cfg = FO.WingConfig(m["nx"], m["ny"], m["nz"], m["chord"], m["x_ea"], m["y_ea"], m["ea"],
                        state=tuple(m["state"]), u0=m["u0"])
    return cfg, z["init/f"]


def fsi_cases():
    from oracle import fsi_oracle as FS
    z, meta = load("fsi_cases")
    for name, m in meta.items():
        keys = ("collision", "nu", "u0", "sponge_start", "sponge_strength", "chord", "x_ea", "y_ea", "ea", "span")
        cfg = FS.FsiConfig(m["nx"], m["ny"], m["nz"], kin=z[f"{name}/kin"], **{k: m[k] for k in keys})
        case = {"name": name, "cfg": cfg, "report": m["report"], "f_in": z[f"{name}/f_in"],
                "f_out": z[f"{name}/f_out"], "solid": z[f"{name}/solid"], "load": z[f"{name}/load"]}
        if m["report"]:
            case["fields"] = {k: z[f"{name}/fields/{k}"] for k in ("ux", "uy", "uz", "p", "vmag")}
        yield case


def derived_cases():
    """Output grids and velocity gradients from the reference's coarsen and _jacobian."""
    z, meta = load("derived_cases")
    for name, m in meta.items():
        case = dict(m, name=name, full={k: z[f"{name}/{k}"] for k in ("ux", "uy", "uz")},
                    out={k: z[f"{name}/out_{k}"] for k in ("ux", "uy", "uz")},
                    jacobian=z[f"{name}/jacobian"])
        yield case
