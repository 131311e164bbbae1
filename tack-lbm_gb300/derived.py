"""Derived fields on the solver's output grid (tack-lbm derived.py, the solver's part).

tack-lbm evaluates VTK-calculator expressions over the output grid with an
external expression compiler (tack-expr, derived.py:20-24); the solver gives
it the velocity and the velocity gradient (``gradient="lattice"``: central
differences on the output grid, one-sided at its faces, derived.py:52-89).
This module provides that gradient and the two default derived fields built
from it (``DEFAULTS``, derived.py:27-30), on the GPU:

* vorticity  = mag(curl(velocity))
* q_criterion = qcrit(velocity) = -1/2 sum_ij du_i/dx_j du_j/dx_i

at points or at cell centres ("@cells": the mean of the eight corner
gradients, the trilinear interpolant at the centre). Other expressions need
the expression compiler and raise ``NotImplementedError``.
"""

import ctypes

DEFAULTS = {
    "vorticity": ("mag(curl(velocity))", "cells"),
    "q_criterion": ("qcrit(velocity)", "cells"),
}
_KNOWN = {"mag(curl(velocity))": "vorticity", "qcrit(velocity)": "q_criterion"}


def parse(specs):
    """'name=expression' or 'name=expression@cells' (default @points) into {name: (expr, at)}
    (derived.py:33-45)."""
    out = {}
    for spec in specs:
        name, _, expr = spec.partition("=")
        if not name or not expr:
            raise SystemExit(f"--derive takes NAME=EXPRESSION[@cells|@points], not {spec!r}")
        at = "points"
        body, sep, where = expr.rpartition("@")
        if sep and where in ("cells", "points"):
            expr, at = body, where
        out[name.strip()] = (expr.strip(), at)
    return out


class DerivedFields:
    """The default derived fields of a Solver's output grid (derived.py:92-128)."""

    def __init__(self, solver, specs=None, gradient="lattice"):
        if gradient != "lattice":
            raise NotImplementedError("only the solver's lattice gradient is provided (gradient='lattice')")
        specs = dict(DEFAULTS if specs is None else specs)
        for name, (expr, at) in specs.items():
            if expr.replace(" ", "") not in _KNOWN or at not in ("points", "cells"):
                raise NotImplementedError(f"{name}: {expr!r} needs the expression compiler; "
                                          "mag(curl(velocity)) and qcrit(velocity) are built in")
        self.solver = solver
        self.specs = specs
        mx, my, mz = solver.out_dims
        self.n = mx * my * mz
        self.inv_h = solver.diameter / solver.stride  # 1 / h, h = stride / diameter (derived.py:101-103)
        self.ncells = max(mx - 1, 0) * max(my - 1, 0) * max(mz - 1, 0)
        from lbm import ManagedArray
        self.jacobian = ManagedArray(9 * self.n)
        self._vort = ManagedArray(max(self.n, self.ncells, 1))
        self._q = ManagedArray(max(self.n, self.ncells, 1))

    @property
    def names(self):
        return list(self.specs)

    def gradient(self):
        """The velocity gradient at the output points, shape (n, 3, 3): [p, c, d] = du_c/dx_d."""
        h = self.solver._h
        h.call("lbm_velocity_gradient", ctypes.c_void_p(self.jacobian.ptr), float(self.inv_h), None)
        h.call("lbm_sync")
        return self.jacobian.numpy[: 9 * self.n].reshape(self.n, 3, 3)

    def evaluate(self):
        """{name: (values, 'vertex' or 'element')} for the current output arrays (derived.py:204-219).
        Both fields of one association come from one pass over the velocity
        (lbm_vorticity_q_direct), with no gradient buffer in between."""
        h = self.solver._h
        done = {}
        results = {}
        for name, (expr, at) in self.specs.items():
            cells = at == "cells"
            m = self.ncells if cells else self.n
            if at not in done:
                h.call("lbm_vorticity_q_direct", float(self.inv_h), ctypes.c_void_p(self._vort.ptr),
                       ctypes.c_void_p(self._q.ptr), int(cells), None)
                h.call("lbm_sync")
                done[at] = (self._vort.numpy[:m].copy(), self._q.numpy[:m].copy())
            vort, q = done[at]
            src = vort if _KNOWN[expr.replace(" ", "")] == "vorticity" else q
            results[name] = (src, "element" if cells else "vertex")
        return results
