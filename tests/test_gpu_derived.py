"""Derived fields on the GPU (derived.py): the output grid's velocity gradient,
vorticity and Q-criterion against the oracle, on the coarsened output grid of
a developing cylinder flow. Tolerance: 1e-5 of the largest value (float32
differences of float32 fields)."""

import numpy as np
import pytest

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
