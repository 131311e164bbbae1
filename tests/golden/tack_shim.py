"""A CPU stand-in for the Tack DSL, used only to generate golden vectors.

The reference solver (tack-lbm ``lbm.py``) is written against Tack, a Python
JIT DSL that is not installed here. Its kernels are ordinary Python functions
whose body is ``for idx in range(lat.n): ...``; Tack compiles them for the GPU,
but as Python they are also a complete, if slow, CPU program. This module
provides just enough of Tack's surface for ``lbm.py`` and ``trt_ref.py`` to
import and execute as plain Python loops:

* ``device_class``, ``func`` and ``kernel`` are identity decorators;
* ``array``/``empty``/``zeros``/``local_array`` return NumPy arrays, with every
  floating-point array promoted to the shim's precision (float64 by default,
  so the reference's arithmetic runs in double precision);
* ``sqrt``/``sin``/``cos`` are injected as globals into the reference module,
  because Tack kernels call them unqualified.

Integer tables (``cx``, ``opp``, ...) are returned as Python lists, which keeps
the interpreted kernels fast enough for grids of a few thousand cells.

This is test infrastructure: nothing in the product imports it.
"""

import math
import sys
import types

import numpy as np

_DTYPE = np.float64


class TArray(np.ndarray):
    """A NumPy array with the ``.numpy()`` accessor Tack arrays expose."""

    def numpy(self):
        return np.asarray(self)


def _wrap(a):
    return np.ascontiguousarray(a).view(TArray)


def make_module(dtype=np.float64):
    """Return a module object that imports as ``tack``."""
    global _DTYPE
    _DTYPE = np.dtype(dtype)
    m = types.ModuleType("tack")
    m.f32 = "f32"
    m.i32 = "i32"

    def ident(obj=None, **_kw):
        if obj is None:
            return lambda o: o
        return obj

    m.device_class = ident
    m.func = ident
    m.kernel = ident

    def array(a, *_, **__):
        a = np.asarray(a)
        if a.dtype.kind in "iu":
            return [int(v) for v in a]
        return _wrap(a.astype(_DTYPE))

    def empty(shape, *_, **__):
        return _wrap(np.full(shape, np.nan, dtype=_DTYPE))

    def zeros(shape, *_, **__):
        return _wrap(np.zeros(shape, dtype=_DTYPE))

    def local_array(_kind, n):
        return np.zeros(n, dtype=_DTYPE)

    def atomic_add(arr, i, v):
        arr[i] += v

    m.array = array
    m.empty = empty
    m.zeros = zeros
    m.local_array = local_array
    m.atomic_add = atomic_add
    m.set_default_device = lambda *_a, **_k: None
    m.sync = lambda: None
    return m


class HostManagedArray:
    """Replacement for the reference's ``ManagedArray`` (lbm.py:525-541).

    The reference allocates CUDA managed memory through cuda-python; here a
    zeroed NumPy array plays both roles (``.numpy`` and ``.tack``).
    """

    def __init__(self, n):
        self.numpy = _wrap(np.zeros(n, dtype=_DTYPE))
        self.tack = self.numpy

    def free(self):
        pass


def import_reference(ref_dir, dtype=np.float64):
    """Import the reference ``lbm`` module from ``ref_dir`` on top of the shim."""
    for name in ("lbm", "tack"):
        sys.modules.pop(name, None)
    sys.modules["tack"] = make_module(dtype)
    if ref_dir not in sys.path:
        sys.path.insert(0, ref_dir)
    import lbm  # noqa: E402  (the reference module)

    lbm.sqrt = math.sqrt
    lbm.sin = math.sin
    lbm.cos = math.cos
    lbm.ManagedArray = HostManagedArray

    # trt_ref.py switches the obstacle off with Cylinder(-100, -100, 0.0). The
    # cylinder's wall velocity divides by the radius (lbm.py:161, lbm.py:165)
    # and the kernel multiplies it by the zero rotation rate and a zero wall
    # flag (lbm.py:422-429): 0 * inf is NaN under IEEE arithmetic and a
    # ZeroDivisionError in Python. A zero radius has no wall at all, so the
    # shim gives it a zero wall velocity.
    vx, vy = lbm.Cylinder.wall_vel_x, lbm.Cylinder.wall_vel_y
    lbm.Cylinder.wall_vel_x = lambda self, x, y, z: 0.0 if self.r == 0 else vx(self, x, y, z)
    lbm.Cylinder.wall_vel_y = lambda self, x, y, z: 0.0 if self.r == 0 else vy(self, x, y, z)
    return lbm
