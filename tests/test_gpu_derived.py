"""Derived fields on the GPU (derived.py): the output grid's velocity gradient,
vorticity and Q-criterion against the oracle, on the coarsened output grid of
a developing cylinder flow, and the output grid and gradient against the
reference's own coarsen and _jacobian (golden fixtures). Tolerance: 1e-5 of
the largest value (float32 differences of float32 fields); against the
golden, each entry within 4 float32 roundings of its own value plus 1e-9 of
the largest (one rounded difference, one rounded scale, float32 inv_h)."""

import ctypes

import numpy as np
import pytest

import goldens
from oracle import lbm_oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("stride", [1, 2])
def test_derived_fields_against_oracle(stride):
    import lbm
    from derived import DEFAULTS, DerivedFields
    s = lbm.Solver(64, 32, 16, collision="les", obstacle="cylinder", reynolds=200.0, u0=0.08,
                   diameter=8.0, stride=stride, init="random", seed=3, rho_sigma=0.0, u_noise=0.01)
    for _ in range(30):
        s.step()
    s.step(report=True)
    s.monitors(31)  # refreshes the output grid
    dims = s.out_dims
    u = [np.asarray(s.output[k].numpy, np.float64) for k in ("ux", "uy", "uz")]
    specs = dict(DEFAULTS)
    specs["vorticity_points"] = ("mag(curl(velocity))", "points")
    specs["q_points"] = ("qcrit(velocity)", "points")
    d = DerivedFields(s, specs)
    g = d.gradient()
    want = O.velocity_gradient(*u, dims, s.diameter / s.stride)
    assert np.abs(g - want).max() <= 1e-5 * np.abs(want).max()
    res = d.evaluate()
    for name, cells in (("vorticity", True), ("q_criterion", True), ("vorticity_points", False),
                        ("q_points", False)):
        w, q = O.vorticity_q(want, dims, cells)
        ref = w if "vort" in name else q
        got, assoc = res[name]
        assert assoc == ("element" if cells else "vertex")
        assert got.shape == ref.shape
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), name
    with pytest.raises(NotImplementedError):
        DerivedFields(s, {"x": ("div(velocity)", "cells")})


@pytest.mark.parametrize("case", list(goldens.derived_cases()), ids=lambda c: c["name"])
def test_derived_gradient_against_reference_golden(case):
    """Fields set through the C ABI, coarsened by lbm_update_output and
    differentiated by lbm_velocity_gradient, against the reference kernels'
    outputs on the same fields: the output grid bit for bit, the gradient to
    float32 rounding."""
    import lbm
    from derived import DerivedFields
    s = lbm.Solver(case["nx"], case["ny"], case["nz"], collision="les", obstacle="cylinder",
                   reynolds=100.0, u0=0.05, diameter=case["diameter"], stride=case["stride"])
    s.sync()
    for k, name in enumerate(("ux", "uy", "uz")):
        v = np.ascontiguousarray(case["full"][name], np.float32)
        s._h.call("lbm_set_field", k, v.ctypes.data_as(ctypes.c_void_p))
    s.update_output()
    s.sync()
    assert tuple(s.out_dims) == tuple(case["out_dims"])
    for name in ("ux", "uy", "uz"):
        assert np.array_equal(s.output[name].numpy, case["out"][name]), name
    g = DerivedFields(s).gradient().reshape(-1, 9).astype(np.float64)
    want = case["jacobian"]
    tol = 4 * 2.0 ** -24 * np.abs(want) + 1e-9 * np.abs(want).max()
    assert (np.abs(g - want) <= tol).all(), np.abs(g - want).max()


@pytest.mark.parametrize("cells", [0, 1])
def test_direct_vorticity_q_equals_gradient_path(cells):
    """lbm_vorticity_q_direct (no gradient buffer) gives the same floats as
    lbm_velocity_gradient followed by lbm_vorticity_q, on an odd-sized output
    grid (one-sided faces on every axis)."""
    import lbm
    s = lbm.Solver(42, 22, 10, collision="les", obstacle="sphere", reynolds=150.0, u0=0.07,
                   diameter=6.0, stride=1, init="random", seed=5, rho_sigma=0.0, u_noise=0.02)
    for _ in range(6):
        s.step()
    s.step(report=True)
    s.monitors(7)
    mx, my, mz = s.out_dims
    n = mx * my * mz
    m = (mx - 1) * (my - 1) * (mz - 1) if cells else n
    inv_h = s.diameter / s.stride
    jac, v1, q1, v2, q2 = (lbm.ManagedArray(k) for k in (9 * n, m, m, m, m))
    h = s._h
    h.call("lbm_velocity_gradient", ctypes.c_void_p(jac.ptr), float(inv_h), None)
    h.call("lbm_vorticity_q", ctypes.c_void_p(jac.ptr), ctypes.c_void_p(v1.ptr), ctypes.c_void_p(q1.ptr),
           cells, None)
    h.call("lbm_vorticity_q_direct", float(inv_h), ctypes.c_void_p(v2.ptr), ctypes.c_void_p(q2.ptr), cells, None)
    h.call("lbm_sync")
    assert np.array_equal(v1.numpy, v2.numpy)
    assert np.array_equal(q1.numpy, q2.numpy)
    assert np.abs(v2.numpy).max() > 0
