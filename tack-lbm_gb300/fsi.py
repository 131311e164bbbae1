"""Fluid-structure interaction of a cantilever wing on the GB300 FSI kernel.

The drop-in for tack-lbm's ``fsi.py``: a 3D flow around an elastic NACA 0012
wing whose root sits on a mirror plane below z = 0 and whose tip is at
z = span, with inflow at x = 0 and an outflow at x = nx - 1. Every step:

* fluid -> structure: each lattice layer's lift and pitching moment by
  momentum exchange (``lbm_fsi_step``), projected on the wing's vibration
  modes as generalized forces;
* structure -> fluid: each layer's plunge and pitch (and their rates) from
  the modal state, through moving-wall bounce-back, second order on wetted
  links (interpolated bounce-back).

The structural model is any object with the modal frequencies ``omega0``,
the modal plunge and twist along the span ``h[k, :]`` and ``alpha[k, :]``
(the last column at the tip) and ``sections_at(z)`` giving the modes'
plunge and twist at heights z. By default it is ``fsi_beam.WingBeam``, the
reference's bending-torsion beam, here assembled with this package's own
1-D finite elements instead of MFEM. ``Modal`` integrates the modal
equations as the reference does.
"""

import ctypes

import numpy as np

import lbm_native as N
from lbm import COLLISIONS, ManagedArray, _host

_OUT = ("ux", "uy", "uz", "p", "vmag")


class FlexWing:
    """NACA 0012 wing from the root plane to ``span`` (fsi.py:25-67); ``kin`` holds
    h, alpha, dh/dt, dalpha/dt per layer (nz, 4); ``load`` receives fx, fy, mz per layer."""

    def __init__(self, chord, x_ea, y_ea, ea, span, kin, load=None):
        self.chord, self.x_ea, self.y_ea, self.ea, self.span = chord, x_ea, y_ea, ea, span
        self.kin = kin
        self.load = np.zeros((len(kin), 3)) if load is None else load


class Modal:
    """Mass-normalised modal dynamics q'' + 2 zeta w q' + w^2 q + dV/dq = Q with a
    quartic torsion potential V = K a^4 / 4, a the tip twist of the whole motion,
    K chosen so the torsion mode alone stiffens as w^2 (1 + H a^2)
    (fsi_struct.py:176-196); semi-implicit Euler."""

    def __init__(self, fem, omega, damping=0.0, hardening=40.0, torsion=1):
        self.fem = fem
        self.omega = np.array(omega, float)
        self.damping, self.hardening, self.torsion = damping, hardening, torsion
        self.tip_twist = np.asarray(fem.alpha[:, -1], float)
        self.q = np.zeros(len(self.omega))
        self.v = np.zeros(len(self.omega))

    def step(self, force, dt=1.0):
        twist = float(self.tip_twist @ self.q)
        k = self.hardening * (self.omega[self.torsion] / self.tip_twist[self.torsion]) ** 2
        restoring = self.omega ** 2 * self.q + k * twist ** 3 * self.tip_twist
        self.v += dt * (force - restoring - 2.0 * self.damping * self.omega * self.v)
        self.q += dt * self.v


def _fsi_config(nx, ny, nz, geo, phys, flow, device):
    c = N.FsiConfig()
    c.nx, c.ny, c.nz = nx, ny, nz
    c.collision = phys.code
    c.nu = phys.nu
    c.cs = getattr(phys, "cs", 0.16)
    c.magic = getattr(phys, "magic", 0.1875)
    c.chord, c.x_ea, c.y_ea, c.ea, c.span = geo.chord, geo.x_ea, geo.y_ea, geo.ea, geo.span
    c.u0, c.sponge_start, c.sponge_strength = flow.u0, flow.sponge_start, flow.sponge_strength
    c.device = device
    return c


class _Handle:
    def __init__(self, cfg):
        self.lib = N.load()
        ptr = ctypes.c_void_p()
        N.check(self.lib.lbm_fsi_create(ctypes.byref(cfg), ctypes.byref(ptr)))
        self.ptr = ptr

    def __del__(self):
        ptr, self.ptr = getattr(self, "ptr", None), None
        if ptr and N._lib is not None:
            N._lib.lbm_fsi_destroy(ptr)

    def call(self, name, *args):
        return N.check(getattr(self.lib, name)(self.ptr, *args))


def _dbl(a):
    v = np.ascontiguousarray(np.asarray(a, np.float64).reshape(-1))
    return v, v.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def fsi_init(lat, geo, flow, f, device=0):
    """fsi_init (fsi.py:71-78) into the host array ``f`` (19*n)."""
    from lbm import BGK
    h = _Handle(_fsi_config(lat.nx, lat.ny, lat.nz, geo, BGK(0.1), flow, device))
    kin, kp = _dbl(geo.kin)
    h.call("lbm_fsi_init", kp)
    out = _host(f)
    buf = np.empty(19 * lat.n, np.float32)
    h.call("lbm_fsi_populations", buf.ctypes.data_as(ctypes.c_void_p), 0)
    out[...] = buf.reshape(out.shape).astype(out.dtype, copy=False)
    return out


def fsi_step(lat, phys, geo, flow, diag, f_in, f_out, device=0):
    """One fsi_step (fsi.py:81-186) from host populations ``f_in`` into ``f_out``;
    ``geo.load`` receives the per-layer (fx, fy, mz), a Report diag the fields."""
    h = _Handle(_fsi_config(lat.nx, lat.ny, lat.nz, geo, phys, flow, device))
    src = np.ascontiguousarray(_host(f_in), dtype=np.float32).reshape(-1)
    h.call("lbm_fsi_populations", src.ctypes.data_as(ctypes.c_void_p), 1)
    report = bool(getattr(diag, "enabled", 0))
    kin, kp = _dbl(geo.kin)
    load = np.zeros(3 * lat.nz)
    h.call("lbm_fsi_step", int(report), kp, load.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    geo.load[...] = load.reshape(lat.nz, 3)
    out = _host(f_out)
    buf = np.empty(19 * lat.n, np.float32)
    h.call("lbm_fsi_populations", buf.ctypes.data_as(ctypes.c_void_p), 0)
    out[...] = buf.reshape(out.shape).astype(out.dtype, copy=False)
    if report:
        for k, name in enumerate(_OUT):
            ptr = ctypes.c_void_p()
            h.call("lbm_fsi_field", k, ctypes.byref(ptr))
            _host(diag.fields[name])[...] = np.ctypeslib.as_array((ctypes.c_float * lat.n).from_address(ptr.value))
    return out


class FSISolver:
    """tack-lbm's FSISolver (fsi.py:189-325) on the GB300 FSI kernel; ``fem``
    defaults to ``fsi_beam.WingBeam(chord, span, ea)`` as there (fsi.py:194)."""

    OUTPUT = _OUT

    def __init__(self, nx=256, ny=128, nz=104, chord=32.0, span=64.0, ea=0.4, u0=0.08, reynolds=500.0,
                 collision="les", reduced_velocity=3.5, damping=0.005, hardening=200.0, device="cuda", stride=1,
                 fem=None):
        from lbm import D3Q19, Flow
        if fem is None:
            from fsi_beam import WingBeam
            fem = WingBeam(chord=chord, span=span, ea=ea)
        self.device_index = 0 if device in ("cuda", None) else int(str(device).split(":")[-1])
        self.nx, self.ny, self.nz = nx, ny, nz
        self.lat = D3Q19(nx, ny, nz)
        self.chord, self.span, self.u0 = chord, span, u0
        self.diameter = chord
        self.flow = Flow(u0, 0.75 * nx, 1.0)
        self.collision_name = collision
        self.set_reynolds(reynolds, _apply=False)
        self.fem = fem
        self.torsion = self._first_torsion()
        self.mode_h, self.mode_alpha = fem.sections_at(np.arange(nz) + 0.5)
        self.structure = Modal(fem, fem.omega0, damping=damping, hardening=hardening, torsion=self.torsion)
        self.stiffness = 1.0
        self.set_reduced_velocity(reduced_velocity)
        self._kin = np.zeros((nz, 4))
        self.geo = FlexWing(chord, 0.25 * nx, 0.5 * ny, ea, span, self._kin)
        self.held = True
        self._h = _Handle(_fsi_config(nx, ny, nz, self.geo, self.phys, self.flow, self.device_index))
        n = self.lat.n
        self.fields = {}
        for k, name in enumerate(_OUT):
            ptr = ctypes.c_void_p()
            self._h.call("lbm_fsi_field", k, ctypes.byref(ptr))
            self.fields[name] = ManagedArray.view(ptr.value, n, self._h)
        self.stride = stride
        self._h.call("lbm_fsi_set_output_stride", int(stride))
        self.out_dims = tuple((d + stride - 1) // stride for d in (nx, ny, nz))
        self.output = {}
        for k, name in enumerate(_OUT):
            ptr, cnt = ctypes.c_void_p(), ctypes.c_int64()
            self._h.call("lbm_fsi_output", k, ctypes.byref(ptr), ctypes.byref(cnt))
            self.output[name] = self.fields[name] if stride == 1 else ManagedArray.view(ptr.value, cnt.value, self._h)
        _, kp = _dbl(self._kin)
        self._h.call("lbm_fsi_init", kp)
        self.step_count = 0
        self.layer_load = np.zeros((nz, 3))
        self.drag = self.lift = self.moment = 0.0

    def _first_torsion(self):
        """The first mode whose tip twist dominates its tip plunge (fsi.py:226-231)."""
        b = 0.5 * self.chord
        for i in range(len(self.fem.omega0)):
            if abs(self.fem.alpha[i, -1]) > abs(self.fem.h[i, -1]) / b and abs(self.fem.alpha[i, -1]) > 0.0:
                return i
        return 1

    def set_reynolds(self, reynolds, _apply=True):
        self.reynolds = float(reynolds)
        self.nu = self.u0 * self.chord / self.reynolds
        self.phys = COLLISIONS[self.collision_name](self.nu)
        if _apply:
            self._h.call("lbm_fsi_set_physics", self.phys.code, float(self.nu))

    def set_physics(self, collision, reynolds):
        """A new air speed at fixed air viscosity and wing: Re and U* scale together (fsi.py:238-244)."""
        speed_ratio = float(reynolds) / self.reynolds
        self.collision_name = collision
        self.set_reynolds(reynolds)
        self.design_omega = self.design_omega / speed_ratio
        self._apply_stiffness()

    def reduced_velocity(self):
        return self.u0 / (0.5 * self.chord * self.structure.omega[self.torsion])

    def set_reduced_velocity(self, value):
        """U* of the first torsion mode at the design stiffness."""
        target = self.u0 / (0.5 * self.chord * value)
        self.design_omega = self.fem.omega0 * (target / self.fem.omega0[self.torsion])
        self._apply_stiffness()

    def set_stiffness(self, fraction):
        """Material stiffness as a fraction of its design value (frequencies scale as its root)."""
        self.stiffness = float(fraction)
        self._apply_stiffness()

    def _apply_stiffness(self):
        self.structure.omega = self.design_omega * np.sqrt(self.stiffness)

    def frequencies(self):
        return self.structure.omega.copy()

    def update_output(self):
        self._h.call("lbm_fsi_update_output")

    def release(self, tip_twist_rate=None):
        """Free the wing, nudged with a twist rate in its first torsion mode (default: a 2 degree tip swing)."""
        self.held = False
        k = self.torsion
        rate = np.radians(2.0) * self.structure.omega[k] if tip_twist_rate is None else tip_twist_rate
        self.structure.v[k] += rate / self.fem.alpha[k, -1]
        self._sync_kinematics()

    def gust(self, degrees):
        """A sudden tip twist rate, as from a gust: the tip swings by about ``degrees``."""
        k = self.torsion
        self.structure.v[k] += np.radians(degrees) * self.structure.omega[k] / self.fem.alpha[k, -1]

    def _sync_kinematics(self):
        s = self.structure
        self._kin[:, 0] = s.q @ self.mode_h
        self._kin[:, 1] = s.q @ self.mode_alpha
        self._kin[:, 2] = s.v @ self.mode_h
        self._kin[:, 3] = s.v @ self.mode_alpha

    def step(self, report=False):
        _, kp = _dbl(self._kin)
        load = np.zeros(3 * self.nz)
        self._h.call("lbm_fsi_step", int(bool(report)), kp, load.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        load = load.reshape(self.nz, 3)
        self.geo.load[...] = load
        load = load.copy()
        load[:, 2] *= -1.0
        self.layer_load = load
        self.drag, self.lift, self.moment = load.sum(0) / self.span
        if not self.held:
            self.structure.step(self.mode_h @ load[:, 1] + self.mode_alpha @ load[:, 2])
            self._sync_kinematics()
        self.step_count += 1

    def populations(self):
        out = np.empty(19 * self.lat.n, np.float32)
        self._h.call("lbm_fsi_populations", out.ctypes.data_as(ctypes.c_void_p), 0)
        return out

    def mask(self):
        out = np.empty(self.lat.n, np.uint8)
        _, kp = _dbl(self._kin)
        self._h.call("lbm_fsi_mask", kp, out.ctypes.data_as(ctypes.c_void_p))
        return out

    def tip(self):
        """Tip plunge in semichords and tip pitch in degrees."""
        k = min(int(self.span - 0.5), self.nz - 1)
        return self._kin[k, 0] / (0.5 * self.chord), np.degrees(self._kin[k, 1])

    def motion(self):
        return self.tip()

    def coefficients(self):
        q = 0.5 * self.u0 * self.u0 * self.chord
        return self.drag / q, self.lift / q, self.moment / (q * self.chord)
