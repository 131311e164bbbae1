"""Pitch-plunge flutter of a NACA 0012 section on the GB300 wing kernel.

The drop-in for tack-lbm's ``flutter.py``: a rigid wing on two springs
(plunge h, up positive; pitch alpha, nose up positive, about the elastic axis
at chord fraction ``ea``), coupled to the flow every lattice step:

* fluid -> structure: lift and pitching moment by momentum exchange on every
  wall link (the GPU kernel ``wing_step_kernel``, ``lbm_wing_step``);
* structure -> fluid: the wing's position and rigid-body velocity through
  bounce-back on a moving wall; cells the wing uncovers start from
  equilibrium at the wall velocity.

The structure (``Section``) is integrated on the host between steps, as the
reference does (flutter.py:134-167). Public names and arguments follow the
reference module; the kernels are this package's sm_103a code.
"""

import ctypes
from math import pi

import numpy as np

import lbm_native as N
from lbm import COLLISIONS, ManagedArray, _host

_OUT = ("ux", "uy", "uz", "p", "vmag")


class Wing:
    """NACA 0012 section spanning z (flutter.py:20-48). ``state`` holds
    (h, alpha, dh/dt, dalpha/dt); ``load`` receives (fx, fy, mz) of the last step."""

    def __init__(self, chord, x_ea, y_ea, ea, state=None, load=None):
        self.chord, self.x_ea, self.y_ea, self.ea = chord, x_ea, y_ea, ea
        self.state = np.zeros(4) if state is None else state
        self.load = np.zeros(3) if load is None else load


class Section:
    """Typical-section structure per unit span at fluid density 1 (flutter.py:134-167):
    mass ratio ``mu``, centre of gravity ``x_alpha`` semichords aft of the elastic
    axis, squared radius of gyration ``r_alpha2`` (semichords^2), frequency ratio
    omega_h / omega_alpha, viscous damping ratio and cubic pitch hardening."""

    def __init__(self, semichord, mu=20.0, x_alpha=0.1, r_alpha2=0.24, freq_ratio=0.4, omega_alpha=0.002,
                 damping=0.0, hardening=0.0):
        self.b, self.mu, self.x_alpha, self.r_alpha2, self.freq_ratio = semichord, mu, x_alpha, r_alpha2, freq_ratio
        self.m = mu * pi * semichord ** 2
        self.damping, self.hardening = damping, hardening
        self.q = np.zeros(2)  # h, alpha
        self.v = np.zeros(2)  # their rates
        self.set_frequency(omega_alpha)

    def set_frequency(self, omega_alpha):
        m, b = self.m, self.b
        self.omega_alpha = omega_alpha
        i_alpha = m * self.r_alpha2 * b * b
        s_alpha = m * self.x_alpha * b
        self.mass = np.array([[m, -s_alpha], [-s_alpha, i_alpha]])
        k_h = m * (self.freq_ratio * omega_alpha) ** 2
        k_alpha = i_alpha * omega_alpha ** 2
        self.stiffness = np.diag([k_h, k_alpha])
        self.dampers = 2.0 * self.damping * np.diag([np.sqrt(k_h * m), np.sqrt(k_alpha * i_alpha)])
        self.inverse = np.linalg.inv(self.mass)

    def step(self, lift, moment, dt=1.0):
        """One semi-implicit Euler step; the pitch spring is k_alpha (alpha + hardening alpha^3)."""
        restoring = self.stiffness @ self.q
        restoring[1] += self.stiffness[1, 1] * self.hardening * self.q[1] ** 3
        accel = self.inverse @ (np.array([lift, moment]) - restoring - self.dampers @ self.v)
        self.v += dt * accel
        self.q += dt * self.v


def _wing_config(nx, ny, nz, geo, phys, flow, device):
    c = N.WingConfig()
    c.nx, c.ny, c.nz = nx, ny, nz
    c.collision = phys.code
    c.nu = phys.nu
    c.cs = getattr(phys, "cs", 0.16)
    c.magic = getattr(phys, "magic", 0.1875)
    c.chord, c.x_ea, c.y_ea, c.ea = geo.chord, geo.x_ea, geo.y_ea, geo.ea
    c.u0, c.sponge_start, c.sponge_strength = flow.u0, flow.sponge_start, flow.sponge_strength
    c.device = device
    return c


class _Handle:
    def __init__(self, cfg):
        self.lib = N.load()
        ptr = ctypes.c_void_p()
        N.check(self.lib.lbm_wing_create(ctypes.byref(cfg), ctypes.byref(ptr)))
        self.ptr = ptr

    def __del__(self):
        ptr, self.ptr = getattr(self, "ptr", None), None
        if ptr and N._lib is not None:
            N._lib.lbm_wing_destroy(ptr)

    def call(self, name, *args):
        return N.check(getattr(self.lib, name)(self.ptr, *args))


def _d4(state):
    return (ctypes.c_double * 4)(*[float(v) for v in np.asarray(state).reshape(4)])


def wing_init(lat, geo, flow, f, device=0):
    """wing_init (flutter.py:51-58) into the host array ``f`` (19*n)."""
    from lbm import BGK
    h = _Handle(_wing_config(lat.nx, lat.ny, lat.nz, geo, BGK(0.1), flow, device))
    h.call("lbm_wing_init", _d4(geo.state))
    out = _host(f)
    buf = np.empty(19 * lat.n, np.float32)
    h.call("lbm_wing_populations", buf.ctypes.data_as(ctypes.c_void_p), 0)
    out[...] = buf.reshape(out.shape).astype(out.dtype, copy=False)
    return out


def wing_step(lat, phys, geo, flow, diag, f_in, f_out, device=0):
    """One wing_step (flutter.py:61-130) from host populations ``f_in`` into ``f_out``;
    ``geo.load`` receives (fx, fy, mz) and a Report diag the fields ux, uy, uz, p, vmag."""
    h = _Handle(_wing_config(lat.nx, lat.ny, lat.nz, geo, phys, flow, device))
    src = np.ascontiguousarray(_host(f_in), dtype=np.float32).reshape(-1)
    h.call("lbm_wing_populations", src.ctypes.data_as(ctypes.c_void_p), 1)
    report = bool(getattr(diag, "enabled", 0))
    load = (ctypes.c_double * 3)()
    h.call("lbm_wing_step", int(report), _d4(geo.state), load)
    geo.load[:] = load[:]
    out = _host(f_out)
    buf = np.empty(19 * lat.n, np.float32)
    h.call("lbm_wing_populations", buf.ctypes.data_as(ctypes.c_void_p), 0)
    out[...] = buf.reshape(out.shape).astype(out.dtype, copy=False)
    if report:
        for k, name in enumerate(_OUT):
            ptr = ctypes.c_void_p()
            h.call("lbm_wing_field", k, ctypes.byref(ptr))
            _host(diag.fields[name])[...] = np.ctypeslib.as_array((ctypes.c_float * lat.n).from_address(ptr.value))
    return out


class FlutterSolver:
    """tack-lbm's FlutterSolver (flutter.py:170-273) on the GB300 wing kernel."""

    OUTPUT = _OUT

    def __init__(self, nx=384, ny=192, nz=4, chord=48.0, ea=0.4, u0=0.08, reynolds=500.0, collision="les",
                 device="cuda", stride=1, **section):
        from lbm import D3Q19, Flow
        self.device_index = 0 if device in ("cuda", None) else int(str(device).split(":")[-1])
        self.nx, self.ny, self.nz = nx, ny, nz
        self.lat = D3Q19(nx, ny, nz)
        self.chord, self.u0 = chord, u0
        self.diameter = chord
        self.flow = Flow(u0, 0.75 * nx, 1.0)
        self.collision_name = collision
        self.set_reynolds(reynolds, _apply=False)
        self.geo = Wing(chord, 0.25 * nx, 0.5 * ny, ea)
        self.section = Section(0.5 * chord, **section)
        self.held = True
        self._h = _Handle(_wing_config(nx, ny, nz, self.geo, self.phys, self.flow, self.device_index))
        n = self.lat.n
        self.fields = {}
        for k, name in enumerate(_OUT):
            ptr = ctypes.c_void_p()
            self._h.call("lbm_wing_field", k, ctypes.byref(ptr))
            self.fields[name] = ManagedArray.view(ptr.value, n, self._h)
        self.stride = stride
        self._h.call("lbm_wing_set_output_stride", int(stride))
        self.out_dims = tuple((d + stride - 1) // stride for d in (nx, ny, nz))
        self.output = {}
        for k, name in enumerate(_OUT):
            ptr, cnt = ctypes.c_void_p(), ctypes.c_int64()
            self._h.call("lbm_wing_output", k, ctypes.byref(ptr), ctypes.byref(cnt))
            self.output[name] = self.fields[name] if stride == 1 else ManagedArray.view(ptr.value, cnt.value, self._h)
        self._h.call("lbm_wing_init", _d4(self.geo.state))
        self.step_count = 0
        self.drag = self.lift = self.moment = 0.0

    def set_reynolds(self, reynolds, _apply=True):
        self.reynolds = float(reynolds)
        self.nu = self.u0 * self.chord / self.reynolds
        self.phys = COLLISIONS[self.collision_name](self.nu)
        if _apply:
            self._h.call("lbm_wing_set_physics", self.phys.code, float(self.nu))

    def set_physics(self, collision, reynolds):
        """A new air speed at fixed air viscosity and wing: Re and U* scale together (flutter.py:212-218)."""
        speed_ratio = float(reynolds) / self.reynolds
        self.collision_name = collision
        self.set_reynolds(reynolds)
        self.set_reduced_velocity(self.reduced_velocity() * speed_ratio)

    def update_output(self):
        self._h.call("lbm_wing_update_output")

    def outline(self, points=96):
        """The section's contour at its current position, as lattice (x, y) (flutter.py:227-240)."""
        beta = np.linspace(0.0, np.pi, points // 2 + 1)
        xc = 0.5 * (1.0 - np.cos(beta))
        half = 0.6 * (0.2969 * np.sqrt(xc) - 0.126 * xc - 0.3516 * xc ** 2 + 0.2843 * xc ** 3 - 0.1036 * xc ** 4)
        xs = np.concatenate([xc[::-1], xc[1:-1]])
        ts = np.concatenate([half[::-1], -half[1:-1]])
        s = (xs - self.geo.ea) * self.chord
        t = ts * self.chord
        h, a = self.section.q
        return (self.geo.x_ea + s * np.cos(a) + t * np.sin(a), self.geo.y_ea + h - s * np.sin(a) + t * np.cos(a))

    def reduced_velocity(self):
        return self.u0 / (self.section.b * self.section.omega_alpha)

    def set_reduced_velocity(self, value):
        self.section.set_frequency(self.u0 / (self.section.b * value))

    def release(self, alpha_rate=None):
        """Free the wing, nudged with a pitch rate (default: a 2 degree swing at omega_alpha)."""
        self.held = False
        self.section.v[1] += np.radians(2.0) * self.section.omega_alpha if alpha_rate is None else alpha_rate
        self._sync_state()

    def _sync_state(self):
        s = self.section
        self.geo.state[:] = (s.q[0], s.q[1], s.v[0], s.v[1])

    def step(self, report=False):
        load = (ctypes.c_double * 3)()
        self._h.call("lbm_wing_step", int(bool(report)), _d4(self.geo.state), load)
        self.geo.load[:] = load[:]
        fx, fy, mz = (v / self.nz for v in load)
        self.drag, self.lift, self.moment = fx, fy, -mz
        if not self.held:
            self.section.step(self.lift, self.moment)
            self._sync_state()
        self.step_count += 1

    def populations(self):
        out = np.empty(19 * self.lat.n, np.float32)
        self._h.call("lbm_wing_populations", out.ctypes.data_as(ctypes.c_void_p), 0)
        return out

    def mask(self):
        out = np.empty(self.lat.n, np.uint8)
        self._h.call("lbm_wing_mask", _d4(self.geo.state), out.ctypes.data_as(ctypes.c_void_p))
        return out

    def coefficients(self):
        q = 0.5 * self.u0 * self.u0 * self.chord
        return self.drag / q, self.lift / q, self.moment / (q * self.chord)

    def motion(self):
        s = self.section
        return s.q[0] / s.b, np.degrees(s.q[1])
