"""GB300 drop-in for tack-lbm's ``lbm`` module (the D3Q19 solver API).

Put this directory on ``sys.path`` and ``from lbm import Solver`` works as with
the reference: the same constructor arguments, ``step``, ``monitors``,
``set_physics``, ``set_obstacle``, ``set_actuation``, ``update_output``, the
managed ``fields`` / ``output`` arrays, and the device-class names and
kernel entry points (``lbm_init``, ``lbm_step``) that scripts such as
``trt_ref.py`` call directly.

Every step runs the hand-written sm_103a kernels of ``liblbm_gb300.so``
through its C ABI (include/lbm_gb300.h, bound in ``lbm_native``). There is no
CPU path: without the library or a GPU, calls raise ``LbmError``.

Differences from the reference, all additive:

* ``storage`` selects the population storage: "f32" (default), "f16"/"bf16"
  (deviations f - w_q) or "f64";
* ``vertical="slip"`` adds free-slip walls in z, ``lateral="lid"`` a moving
  no-slip wall above y = ny-1 (velocity ``u_lid``);
* ``cs``, ``obstacle_center``, ``obstacle_size`` and ``sponge_start`` /
  ``sponge_planes`` / ``sponge_strength`` override the reference's fixed
  values (lbm.py:107, lbm.py:561, lbm.py:628-637), which stay the defaults;
* ``kernel="bulkcopy"`` selects the bulk-copy (TMA) staged step kernel
  instead of the default per-cell one;
* populations are updated in place (AA pattern): ``f`` is a one-element list
  holding the current populations in the reference layout, read back from
  the GPU.
"""

import ctypes

import numpy as np

import lbm_native as N
from lbm_native import LbmError  # noqa: F401  (re-exported)

CX = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
CY = [0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1]
CZ = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1]
W = [1 / 3] + [1 / 18] * 6 + [1 / 36] * 12

# D3Q7 for temperature: rest plus the six faces, c_s^2 = 1/4 (lbm.py:20-25)
CX7 = [0, 1, -1, 0, 0, 0, 0]
CY7 = [0, 0, 0, 1, -1, 0, 0]
CZ7 = [0, 0, 0, 0, 0, 1, -1]
W7 = [1 / 4] + [1 / 8] * 6
OPP7 = [0, 2, 1, 4, 3, 6, 5]
FIELDS = N.FIELDS


def _opposite():
    return [next(p for p in range(19) if (CX[p], CY[p], CZ[p]) == (-CX[q], -CY[q], -CZ[q]))
            for q in range(19)]


def _mirror_y():
    return [next(p for p in range(19) if (CX[p], CY[p], CZ[p]) == (CX[q], -CY[q], CZ[q]))
            for q in range(19)]


def _host(a):
    """A NumPy view of an array argument (NumPy array or anything with .numpy())."""
    if hasattr(a, "numpy") and callable(a.numpy):
        a = a.numpy()
    elif hasattr(a, "numpy"):
        a = a.numpy
    return a


# ---------------------------------------------------------------------------
# Device classes: the reference composes its kernel from these (lbm.py:38-380);
# here they are plain descriptions turned into an lbm_config.

class D3Q19:
    Q = 19

    def __init__(self, nx, ny, nz):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.n = nx * ny * nz
        self.cx = np.array(CX, np.int32)
        self.cy = np.array(CY, np.int32)
        self.cz = np.array(CZ, np.int32)
        self.w = np.array(W, np.float32)
        self.opp = np.array(_opposite(), np.int32)
        self.miry = np.array(_mirror_y(), np.int32)

    def feq(self, q, rho, ux, uy, uz):
        cu = 3.0 * (float(self.cx[q]) * ux + float(self.cy[q]) * uy + float(self.cz[q]) * uz)
        return self.w[q] * rho * (1.0 + cu + 0.5 * cu * cu - 1.5 * (ux * ux + uy * uy + uz * uz))


class BGK:
    code = N.BGK
    cs = 0.16

    def __init__(self, nu):
        self.nu = nu
        self.omega = 1.0 / (3.0 * nu + 0.5)


class TRT:
    """Two-relaxation-time collision with a Smagorinsky subgrid viscosity (lbm.py:96-123)."""

    code = N.TRT
    magic = 0.1875
    cs = 0.16

    def __init__(self, nu, cs=None):
        self.nu = nu
        self.tau0 = 3.0 * nu + 0.5
        if cs is not None:
            self.cs = cs


class SmagorinskyLES:
    code = N.LES
    cs = 0.16

    def __init__(self, nu, cs=None):
        self.nu = nu
        self.tau0 = 3.0 * nu + 0.5
        if cs is not None:
            self.cs = cs


class Cylinder:
    code = N.CYLINDER

    def __init__(self, x, y, r):
        self.x, self.y, self.r = x, y, r

    def geometry(self):
        return [self.x, self.y, 0.0, self.r, 0.0, 0.0, 0.0]


class Sphere:
    code = N.SPHERE

    def __init__(self, x, y, z, r):
        self.x, self.y, self.z, self.r = x, y, z, r

    def geometry(self):
        return [self.x, self.y, self.z, self.r, 0.0, 0.0, 0.0]


class Box:
    code = N.BOX

    def __init__(self, x, y, z, hx, hy, hz):
        self.x, self.y, self.z = x, y, z
        self.hx, self.hy, self.hz = hx, hy, hz

    def geometry(self):
        return [self.x, self.y, self.z, 0.0, self.hx, self.hy, self.hz]


class NoObstacle:
    code = N.NO_OBSTACLE

    def geometry(self):
        return [0.0] * 7


class HeatSink:
    """A finned heat sink on the floor of a duct (lbm.py:230-276): base plate and
    fins along x, duct walls at y = 0 and y = ny - 1. Sizes in lattice cells."""

    code = N.HEATSINK

    def __init__(self, ny, x0, length, z0, width, base, fin_height, fin_thickness, fin_pitch):
        self.ny = ny
        self.params = [float(v) for v in (x0, length, z0, width, base, fin_height, fin_thickness, fin_pitch)]

    def geometry(self):
        return [0.0] * 7

    def sink_params(self):
        return list(self.params)


class PeriodicY:
    code = N.PERIODIC


class SlipY:
    """Free-slip walls halfway outside y = 0 and y = ny - 1 (lbm.py:355-369)."""

    code = N.SLIP


class LidY:
    """Free-slip wall below y = 0, no-slip wall above y = ny - 1 moving at (u_lid, 0, 0)."""

    code = N.LID

    def __init__(self, u_lid=0.0):
        self.u_lid = u_lid


class PeriodicZ:
    code = N.PERIODIC


class SlipZ:
    code = N.SLIP


class Flow:
    def __init__(self, u0, sponge_start, sponge_strength, omega_rot=None, side=None, vertical=None):
        self.u0 = u0
        self.sponge_start = sponge_start
        self.sponge_strength = sponge_strength
        self.omega_rot = np.zeros(1, np.float32) if omega_rot is None else omega_rot
        self.side = PeriodicY() if side is None else side
        self.vertical = PeriodicZ() if vertical is None else vertical

    def rotation(self):
        v = _host(self.omega_rot)
        return float(np.asarray(v).reshape(-1)[0]) if not np.isscalar(v) else float(v)


class NoHeat:
    """The disabled thermal variant (lbm.py:282-308)."""

    enabled = 0
    Q = 7
    pr_t = 0.85

    def __init__(self, arrays=None):
        self.arrays = arrays or {}
        self.alpha = 0.0
        self.nu = 0.0


class Heat(NoHeat):
    """D3Q7 temperature (lbm.py:311-319): ``arrays`` holds ``t_solid``,
    ``q_solid`` and ``temp`` (length n); ``alpha`` is the molecular diffusivity,
    ``nu`` the viscosity the subgrid diffusivity subtracts."""

    enabled = 1

    def __init__(self, arrays, alpha, nu):
        super().__init__(arrays)
        self.alpha = alpha
        self.nu = nu


class Quiet:
    enabled = 0

    def __init__(self, fields):
        self.fields = fields


class Report(Quiet):
    enabled = 1


class _ManagedBlock:
    """Frees one lbm_managed_alloc allocation when the last view goes away."""

    def __init__(self, address):
        self.address = address

    def __del__(self):
        if self.address and N._lib is not None:
            N._lib.lbm_managed_free(ctypes.c_void_p(self.address))
            self.address = None


class ManagedArray:
    """A CUDA managed float32 array seen as a NumPy array (lbm.py:525-541).

    ``ManagedArray(n)`` allocates n zeroed floats, as the reference does;
    arrays owned by a solver are views created with ``ManagedArray.view``.
    The NumPy view keeps the memory alive. ``tack`` is the same view (there is
    no Tack array type here).
    """

    def __init__(self, n):
        lib = N.load()
        ptr = ctypes.c_void_p()
        N.check(lib.lbm_managed_alloc(int(n), ctypes.byref(ptr)))
        self._setup(ptr.value, n, _ManagedBlock(ptr.value))

    @classmethod
    def view(cls, address, n, owner):
        obj = cls.__new__(cls)
        obj._setup(address, n, owner)
        return obj

    def _setup(self, address, n, owner):
        buf = (ctypes.c_float * n).from_address(address)
        buf._owner = owner
        self.ptr = address
        self.numpy = np.ctypeslib.as_array(buf)
        self.tack = self.numpy

    def free(self):
        """Kept for API parity; the memory is released with the last view."""


COLLISIONS = {"bgk": BGK, "trt": TRT, "les": SmagorinskyLES}


def _config(lat, phys, geo, flow, storage="f32", device=0, heat=None):
    c = N.Config()
    c.nx, c.ny, c.nz = lat.nx, lat.ny, lat.nz
    c.collision = phys.code
    c.obstacle = geo.code
    c.lateral = flow.side.code
    c.vertical = flow.vertical.code
    c.storage = N.STORAGE[storage]
    c.nu = phys.nu
    c.cs = getattr(phys, "cs", 0.16)
    c.magic = getattr(phys, "magic", 0.1875)
    c.ox, c.oy, c.oz, c.r, c.hx, c.hy, c.hz = (float(v) for v in geo.geometry())
    c.u0 = flow.u0
    c.sponge_start = flow.sponge_start
    c.sponge_strength = flow.sponge_strength
    c.u_lid = getattr(flow.side, "u_lid", 0.0)
    c.omega_rot = flow.rotation()
    c.device = device
    if hasattr(geo, "sink_params"):
        c.sink[:] = geo.sink_params()
    if heat is not None and getattr(heat, "enabled", 0):
        c.heat = 1
        c.alpha = float(heat.alpha)
        c.heat_nu = float(heat.nu)
    return c


def lbm_init(lat, geo, flow, f, seed_amp, storage="f32", device=0):
    """The reference's init kernel (lbm.py:383-394) into the host array ``f`` (19*n)."""
    h = N.Handle(_config(lat, BGK(0.1), geo, flow, storage, device))
    h.call("lbm_init", float(seed_amp))
    out = _host(f)
    buf = np.empty(19 * lat.n, np.float64)
    h.call("lbm_get_populations", buf.ctypes.data_as(ctypes.c_void_p), N.F64, N.HOST)
    out[...] = buf.reshape(out.shape).astype(out.dtype, copy=False)
    return out


def _heat_view(h, k, n):
    ptr = ctypes.c_void_p()
    h.call("lbm_heat_field", k, ctypes.byref(ptr))
    return np.ctypeslib.as_array((ctypes.c_float * n).from_address(ptr.value))


def lbm_step(lat, phys, geo, flow, diag, f_in, f_out, heat=None, g_in=None, g_out=None,
             storage="f32", device=0):
    """One step from host populations ``f_in`` into ``f_out`` (the reference's
    kernel signature, lbm.py:397-398). With a ``Report`` diag the 13 fields of
    ``diag.fields`` are read (previous ux, uy, uz, p) and rewritten. With an
    enabled ``Heat`` the temperature populations go from ``g_in`` to ``g_out``
    (7*n), ``heat.arrays["t_solid"]`` is read and, on report steps,
    ``temp`` is written and ``q_solid`` accumulated (lbm.py:457-492)."""
    heat_on = heat is not None and getattr(heat, "enabled", 0)
    h = N.Handle(_config(lat, phys, geo, flow, storage, device, heat))
    src = np.ascontiguousarray(_host(f_in), dtype=np.float64).reshape(-1)
    h.call("lbm_set_populations", src.ctypes.data_as(ctypes.c_void_p), N.F64, N.HOST)
    report = bool(getattr(diag, "enabled", 0))
    if report:
        for k, name in enumerate(N.FIELDS):
            v = np.ascontiguousarray(_host(diag.fields[name]), dtype=np.float32)
            h.call("lbm_set_field", k, v.ctypes.data_as(ctypes.c_void_p))
    if heat_on:
        gsrc = np.ascontiguousarray(_host(g_in), dtype=np.float64).reshape(-1)
        h.call("lbm_set_heat_populations", gsrc.ctypes.data_as(ctypes.c_void_p), N.F64, N.HOST)
        h.call("lbm_sync")
        _heat_view(h, 0, lat.n)[...] = np.asarray(_host(heat.arrays["t_solid"]), np.float32).reshape(-1)
    if heat_on and report:
        # the reference accumulates into q_solid (the caller zeroes it); the
        # library zeroes it first, so add the caller's values back afterwards
        q_before = np.asarray(_host(heat.arrays["q_solid"]), np.float32).reshape(-1).copy()
    h.call("lbm_step", int(report), None)
    out = _host(f_out)
    buf = np.empty(19 * lat.n, np.float64)
    h.call("lbm_get_populations", buf.ctypes.data_as(ctypes.c_void_p), N.F64, N.HOST)
    out[...] = buf.reshape(out.shape).astype(out.dtype, copy=False)
    if report:
        h.call("lbm_sync")
        for k, name in enumerate(N.FIELDS):
            ptr = ctypes.c_void_p()
            h.call("lbm_field", k, ctypes.byref(ptr))
            vals = np.ctypeslib.as_array((ctypes.c_float * lat.n).from_address(ptr.value))
            _host(diag.fields[name])[...] = vals
    if heat_on:
        gbuf = np.empty(7 * lat.n, np.float64)
        h.call("lbm_get_heat_populations", gbuf.ctypes.data_as(ctypes.c_void_p), N.F64, N.HOST)
        gout = _host(g_out)
        gout[...] = gbuf.reshape(gout.shape).astype(gout.dtype, copy=False)
        if report:
            h.call("lbm_sync")
            _host(heat.arrays["temp"])[...] = _heat_view(h, 2, lat.n)
            _host(heat.arrays["q_solid"])[...] = _heat_view(h, 1, lat.n) + q_before
    return out


# ---------------------------------------------------------------------------

class Solver:
    """tack-lbm's Solver (lbm.py:548-661) on the GB300 kernels."""

    OUTPUT = ("ux", "uy", "uz", "p", "vmag")

    def __init__(self, nx=384, ny=128, nz=64, collision="les", obstacle="cylinder",
                 reynolds=300.0, u0=0.08, diameter=24.0, device="cuda", stride=1,
                 heat=False, prandtl=0.7, lateral="periodic", *, storage="f32",
                 vertical="periodic", cs=None, obstacle_center=None, obstacle_size=None,
                 sponge_start=None, sponge_planes=None, sponge_strength=1.0, u_lid=0.0,
                 init="wave", seed=0, rho_sigma=1e-3, u_noise=0.01, kernel="auto"):
        self.device_index = 0 if device in ("cuda", None) else int(str(device).split(":")[-1])
        self.lateral = lateral
        self.vertical_policy = vertical
        self.storage = storage
        self.nx, self.ny, self.nz = nx, ny, nz
        self.lat = D3Q19(nx, ny, nz)
        self.u0, self.diameter = u0, diameter
        self.step_count = 0
        self.heat_enabled = bool(heat)
        self.prandtl = prandtl
        self._cs = cs
        self._obstacle_center = obstacle_center
        self._obstacle_size = obstacle_size
        if sponge_planes is not None:
            sponge_start = nx - sponge_planes
        side = {"periodic": PeriodicY, "slip": SlipY, "lid": lambda: LidY(u_lid)}[lateral]()
        vert = {"periodic": PeriodicZ, "slip": SlipZ}[vertical]()
        self.flow = Flow(u0, 0.75 * nx if sponge_start is None else sponge_start, sponge_strength,
                         np.zeros(1, np.float32), side, vert)
        self.set_obstacle(obstacle, _apply=False)
        self.set_physics(collision, reynolds, _apply=False)
        n = self.lat.n
        if self.heat_enabled:
            # Heat(arrays, nu / prandtl, nu) at construction (lbm.py:596-599)
            self.heat = Heat({}, self.nu / self.prandtl, self.nu)
        else:
            self.heat = NoHeat()
        cfg = _config(self.lat, self.phys, self.geo, self.flow, storage, self.device_index, self.heat)
        cfg.flags = {"auto": 0, "bulkcopy": N.FLAG_BULKCOPY, "simt": N.FLAG_SIMT}[kernel]
        self._h = N.Handle(cfg)
        self._setup_heat(n)
        self.fields = {}
        for k, name in enumerate(FIELDS):
            ptr = ctypes.c_void_p()
            self._h.call("lbm_field", k, ctypes.byref(ptr))
            self.fields[name] = ManagedArray.view(ptr.value, n, self._h)
        self.stride = stride
        self.out_dims = tuple((d + stride - 1) // stride for d in (nx, ny, nz))
        self._h.call("lbm_set_output_stride", int(stride))
        self.output = {}
        outputs = self.OUTPUT + (("temp",) if self.heat_enabled else ())
        for k, name in enumerate(outputs):
            ptr, cnt = ctypes.c_void_p(), ctypes.c_int64()
            self._h.call("lbm_output", k, ctypes.byref(ptr), ctypes.byref(cnt))
            full = self.heat_fields[name] if name == "temp" else self.fields.get(name)
            self.output[name] = full if stride == 1 else ManagedArray.view(ptr.value, cnt.value, self._h)
        if init == "wave":
            self._h.call("lbm_init", 0.05)
        elif init == "random":
            self._h.call("lbm_init_random", float(rho_sigma), float(u_noise), int(seed))
        else:
            raise KeyError(init)
        self.step(report=True)
        self.step_count = 0

    def _setup_heat(self, n):
        """The temperature fields t_solid, q_solid, temp (lbm.py:586-600): managed
        arrays of n floats when the run has heat, empty otherwise."""
        self.heat_fields = {}
        if self.heat_enabled:
            for k, name in enumerate(N.HEAT_FIELDS):
                ptr = ctypes.c_void_p()
                self._h.call("lbm_heat_field", k, ctypes.byref(ptr))
                self.heat_fields[name] = ManagedArray.view(ptr.value, n, self._h)
            self.heat.arrays = {k: v.numpy for k, v in self.heat_fields.items()}

    def set_wall_temperature(self, value):
        """Fill every solid voxel's temperature (lbm.py:602-604)."""
        self.sync()
        self.heat_fields["t_solid"].numpy[:] = value

    @property
    def g(self):
        """The current temperature populations g[q*n + idx] (7*n), in a one-element list."""
        if not self.heat_enabled:
            return [None]
        out = np.empty(7 * self.lat.n, np.float32)
        self._h.call("lbm_get_heat_populations", out.ctypes.data_as(ctypes.c_void_p), N.F32, N.HOST)
        return [out]

    def set_heat_populations(self, g):
        src = np.ascontiguousarray(_host(g), dtype=np.float64).reshape(-1)
        if src.size != 7 * self.lat.n:
            raise ValueError("temperature populations must hold 7*n values")
        self._h.call("lbm_set_heat_populations", src.ctypes.data_as(ctypes.c_void_p), N.F64, N.HOST)

    # -- composition ------------------------------------------------------
    def set_physics(self, collision, reynolds, _apply=True):
        self.collision_name, self.reynolds = collision, float(reynolds)
        self.nu = self.u0 * self.diameter / self.reynolds
        self.phys = COLLISIONS[collision](self.nu)
        if self._cs is not None:
            self.phys.cs = self._cs
        if _apply:
            self._h.call("lbm_set_physics", self.phys.code, float(self.nu), float(self.phys.cs))

    def set_obstacle(self, kind, _apply=True):
        nx, ny, nz, r = self.nx, self.ny, self.nz, self.diameter / 2
        x0, y0 = 0.22 * nx, 0.5 * ny + 1.7
        z0 = 0.5 * nz
        if self._obstacle_center is not None:
            x0, y0, z0 = self._obstacle_center
        size = self._obstacle_size
        self.obstacle_name = kind
        if kind == "cylinder":
            geo = Cylinder(x0, y0, r if size is None else size)
        elif kind == "sphere":
            geo = Sphere(x0, y0, z0, r if size is None else size)
        elif kind == "box":
            hx, hy, hz = (r, r, 0.3 * nz) if size is None else size
            geo = Box(x0, y0, z0, hx, hy, hz)
        elif kind == "heatsink":
            d = self.diameter
            geo = HeatSink(ny, int(0.2 * nx), int(0.3 * nx), int(0.125 * nz), int(0.75 * nz), round(d / 2),
                           int(0.45 * ny), round(d / 3), round(d))
        elif kind == "none":
            geo = NoObstacle()
        else:
            raise KeyError(kind)
        self.geo = geo
        if _apply:
            if kind == "heatsink":
                self._h.call("lbm_set_sink", (ctypes.c_double * 8)(*geo.sink_params()))
            g = (ctypes.c_double * 7)(*geo.geometry())
            self._h.call("lbm_set_obstacle", geo.code, g)

    def set_actuation(self, omega_rot):
        """Set the cylinder surface speed in lattice units (alpha * u0)."""
        self.flow.omega_rot[0] = float(omega_rot)
        self._h.call("lbm_set_actuation", float(omega_rot))

    @property
    def omega_rot(self):
        return float(self.flow.omega_rot[0])

    def set_sponge(self, start=None, strength=None):
        if start is not None:
            self.flow.sponge_start = start
        if strength is not None:
            self.flow.sponge_strength = strength
        self._h.call("lbm_set_sponge", float(self.flow.sponge_start), float(self.flow.sponge_strength))

    # -- stepping ---------------------------------------------------------
    def step(self, report=False, stream=None):
        self._h.call("lbm_step", int(bool(report)), stream)
        self.step_count += 1

    def run(self, steps, report_last=False, stream=None):
        """``steps`` steps in one native call, the last one a report step if asked."""
        self._h.call("lbm_run", int(steps), int(bool(report_last)), stream)
        self.step_count += steps

    def update_output(self):
        self._h.call("lbm_update_output", None)

    def read_output(self, out):
        """Copy the output fields into the host arrays ``out[name]`` (float32,
        C-contiguous, ideally pinned) with one copy-engine transfer each, then
        wait for them: a host copy instead of reading the managed fields in place."""
        for k, name in enumerate(self.output):
            if name in out:
                a = out[name]
                if a.dtype != np.float32 or not a.flags.c_contiguous or a.size != self.output[name].numpy.size:
                    raise ValueError(f"out[{name!r}] must be a C-contiguous float32 array of the output size")
                self._h.call("lbm_read_output", k, a.ctypes.data_as(ctypes.c_void_p), None)
        self.sync()

    def monitors(self, interval):
        self.update_output()
        out = (ctypes.c_double * 7)()
        self._h.call("lbm_monitors", int(interval), float(self.diameter), out, allow=(N.ERR_NONFINITE,))
        return dict(zip(N.MONITORS, list(out)))

    def field_sums(self):
        out = (ctypes.c_double * 8)()
        self._h.call("lbm_field_sums", out)
        return list(out)

    def sync(self):
        self._h.call("lbm_sync")

    # -- state ------------------------------------------------------------
    def populations(self, dtype=np.float32):
        """The current populations in the reference layout f[q*n + idx]."""
        dt = np.dtype(dtype)
        out = np.empty(19 * self.lat.n, dt)
        code = N.F64 if dt == np.float64 else N.F32
        self._h.call("lbm_get_populations", out.ctypes.data_as(ctypes.c_void_p), code, N.HOST)
        return out

    def set_populations(self, f):
        src = np.ascontiguousarray(_host(f), dtype=np.float64).reshape(-1)
        if src.size != 19 * self.lat.n:
            raise ValueError("populations must hold 19*n values")
        self._h.call("lbm_set_populations", src.ctypes.data_as(ctypes.c_void_p), N.F64, N.HOST)

    @property
    def f(self):
        return [self.populations()]

    def mask(self):
        out = np.empty(self.lat.n, np.uint8)
        self._h.call("lbm_mask", out.ctypes.data_as(ctypes.c_void_p))
        return out

    def memory_bytes(self):
        v = ctypes.c_int64()
        self._h.call("lbm_memory", ctypes.byref(v))
        return v.value
