"""The C ABI library without a GPU: it loads, exports every declared entry
point, its struct layout matches the header, and argument errors come back as
status codes (no compute call is made)."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lbm_gb300.h")


@pytest.fixture(scope="module")
def N():
    import lbm_native as N
    N.load()
    return N


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:lbm_status|int32_t|const char \*)\s*(lbm_\w+)\(", text, re.M)))


def test_every_declared_symbol_is_exported(N):
    names = declared()
    assert len(names) >= 25
    lib = N.load()
    for name in names:
        assert hasattr(lib, name), name
        assert name in N._SIGNATURES, f"{name} has no ctypes signature"


def test_abi_version(N):
    assert N.load().lbm_abi_version() == 2


def test_config_layout(N):
    # 8 int32, 15 doubles, 2 int32, 8 doubles, 2 int32, 2 doubles
    # (include/lbm_gb300.h struct lbm_config)
    assert ctypes.sizeof(N.Config) == 8 * 4 + 15 * 8 + 2 * 4 + 8 * 8 + 2 * 4 + 2 * 8
    assert N.Config.nu.offset == 32
    assert N.Config.device.offset == 32 + 15 * 8
    assert N.Config.sink.offset == 32 + 15 * 8 + 8
    assert N.Config.heat_nu.offset == 32 + 15 * 8 + 8 + 64 + 8 + 8


def base_config(N):
    c = N.Config()
    c.nx, c.ny, c.nz = 16, 8, 4
    c.collision, c.obstacle, c.storage = N.LES, N.CYLINDER, N.F32
    c.nu, c.cs, c.magic, c.r, c.u0 = 0.01, 0.16, 0.1875, 2.0, 0.05
    c.sponge_start, c.sponge_strength = 12.0, 1.0
    return c


@pytest.mark.parametrize("field,value", [
    ("collision", 7), ("obstacle", 9), ("lateral", 5), ("vertical", 2), ("storage", 11),
    ("nx", 0), ("nu", 0.0), ("nu", float("nan")), ("cs", -1.0), ("u0", float("inf")),
    ("alpha", -1.0), ("storage_with_heat", 1)])
def test_invalid_config_is_an_argument_error(N, field, value):
    """Unknown models and bad sizes are rejected before any device work
    (the reference raises KeyError, lbm.py:616, lbm.py:632-637)."""
    c = base_config(N)
    if field in ("alpha", "storage_with_heat"):
        c.heat = 1
        field = "storage" if field == "storage_with_heat" else field
    setattr(c, field, value)
    ptr = ctypes.c_void_p()
    status = N.load().lbm_create(ctypes.byref(c), ctypes.byref(ptr))
    assert status == N.ERR_ARG
    assert N.load().lbm_last_error()
    assert not ptr.value


def test_null_arguments(N):
    lib = N.load()
    assert lib.lbm_create(None, None) == N.ERR_ARG
    assert lib.lbm_step(None, 0, None) == N.ERR_ARG
    assert lib.lbm_destroy(None) == N.OK
    assert lib.lbm_managed_alloc(0, ctypes.byref(ctypes.c_void_p())) == N.ERR_ARG


def test_python_api_surface():
    """The drop-in module exposes the reference module's public names (lbm.py)."""
    import lbm
    for name in ("CX", "CY", "CZ", "W", "D3Q19", "BGK", "TRT", "SmagorinskyLES", "Cylinder", "Sphere",
                 "Box", "PeriodicY", "SlipY", "Flow", "Quiet", "Report", "NoHeat", "ManagedArray",
                 "COLLISIONS", "FIELDS", "Solver", "lbm_init", "lbm_step", "_opposite", "_mirror_y"):
        assert hasattr(lbm, name), name
    for meth in ("step", "monitors", "set_physics", "set_obstacle", "set_actuation", "update_output"):
        assert callable(getattr(lbm.Solver, meth))
    assert isinstance(lbm.Solver.omega_rot, property)
    assert lbm.FIELDS == ("ux", "uy", "uz", "p", "vmag", "r_rho", "r_ux", "r_uy", "r_uz", "r_ke",
                          "fx", "fy", "fz")
