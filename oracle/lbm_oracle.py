"""CPU oracle for the D3Q19 stream-and-collide step (test infrastructure only).

This module restates, in vectorised NumPy, the arithmetic of tack-lbm's GPU
step so that the CUDA kernels can be checked against it. It is the checker,
never the product: only the tests, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` may import it.

Every function cites the reference lines it follows (paths inside the
tack-lbm project). The arithmetic order mirrors the reference so that, in
float64, the oracle reproduces the reference kernel executed as Python (see
``tests/golden/make_golden.py``) to round-off.

Reference anchors
-----------------
* lattice tables ``CX, CY, CZ, W``, opposite / y-mirror: ``lbm.py:15-18``, ``lbm.py:28-35``.
  ``W`` is uploaded as float32 (``lbm.py:48``), so the weights used here are the
  float32-rounded values.
* ``feq``: ``lbm.py:52-55``.
* collisions ``BGK`` / ``smagorinsky_tau`` / ``TRT`` / ``SmagorinskyLES``: ``lbm.py:60-139``.
* obstacles ``Cylinder`` / ``Sphere`` / ``Box``: ``lbm.py:144-227``.
* lateral policies ``PeriodicY`` / ``SlipY``: ``lbm.py:342-369``.
* ``lbm_init``: ``lbm.py:383-394``; ``lbm_step``: ``lbm.py:397-456`` and ``lbm.py:493-513``.
* ``Solver.monitors``: ``lbm.py:649-661``; obstacle placement ``lbm.py:628-637``.

Extensions that the reference does not have (each defaults to the reference
behaviour): a runtime Smagorinsky constant ``cs`` (the reference fixes 0.16,
``lbm.py:107``, ``lbm.py:128``); an explicit obstacle placement; free-slip
walls in z (``vertical="slip"``, the z analogue of ``SlipY``); and a
``lateral="lid"`` policy with a free-slip wall below y = 0 and a no-slip wall
above y = ny - 1 moving with velocity ``(u_lid, 0, 0)``, applied by halfway
bounce-back with the same moving-wall term as the cylinder (``lbm.py:426-428``).
The lid is not part of the obstacle, so it adds nothing to the force fields.
"""

from dataclasses import dataclass, field, replace

import numpy as np

CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1])
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, np.float32).astype(np.float64)


def _table(flip):
    c = np.stack([CX, CY, CZ], 1)
    return np.array([int(np.flatnonzero((c == c[q] * flip).all(1))[0]) for q in range(19)])


OPP = _table(np.array([-1, -1, -1]))
MIRY = _table(np.array([1, -1, 1]))
MIRZ = _table(np.array([1, 1, -1]))

FIELDS = ("ux", "uy", "uz", "p", "vmag", "r_rho", "r_ux", "r_uy", "r_uz", "r_ke", "fx", "fy", "fz")

# D3Q7 for temperature (lbm.py:20-25): rest plus the six faces, float32 weights
CX7 = np.array([0, 1, -1, 0, 0, 0, 0])
CY7 = np.array([0, 0, 0, 1, -1, 0, 0])
CZ7 = np.array([0, 0, 0, 0, 0, 1, -1])
W7 = np.array([1 / 4] + [1 / 8] * 6, np.float32).astype(np.float64)
OPP7 = np.array([0, 2, 1, 4, 3, 6, 5])
PR_T = 0.85  # turbulent Prandtl number (lbm.py:285)
HEAT_FIELDS = ("t_solid", "q_solid", "temp")


@dataclass
class Config:
    """One run configuration: the union of the reference's device classes."""

    nx: int
    ny: int
    nz: int
    collision: str = "les"          # "bgk" | "trt" | "les"
    nu: float = 0.0064
    cs: float = 0.16                # Smagorinsky constant (TRT and LES)
    magic: float = 0.1875           # TRT magic parameter (lbm.py:106)
    obstacle: str = "cylinder"      # "cylinder" | "sphere" | "box" | "none"
    ox: float = 0.0                 # obstacle centre
    oy: float = 0.0
    oz: float = 0.0
    r: float = 0.0                  # cylinder / sphere radius
    hx: float = 0.0                 # box half sizes
    hy: float = 0.0
    hz: float = 0.0
    u0: float = 0.08
    sponge_start: float = 0.0
    sponge_strength: float = 1.0
    omega_rot: float = 0.0
    lateral: str = "periodic"       # "periodic" | "slip" | "lid"
    vertical: str = "periodic"      # "periodic" | "slip"
    u_lid: float = 0.0
    # HeatSink (lbm.py:230-276): x0, length, z0, width, base, fin_height,
    # fin_thickness, fin_pitch, in cells
    sink: tuple = (0, 0, 0, 0, 0, 0, 1, 1)
    # D3Q7 temperature (lbm.py:279-319, lbm.py:457-492)
    heat: bool = False
    alpha: float = 0.0              # molecular diffusivity (nu / prandtl at construction)
    heat_nu: float = 0.0            # the viscosity the subgrid diffusivity subtracts

    @property
    def n(self):
        return self.nx * self.ny * self.nz


def solver_config(nx=384, ny=128, nz=64, collision="les", obstacle="cylinder", reynolds=300.0,
                  u0=0.08, diameter=24.0, lateral="periodic", **extra):
    """The configuration ``lbm.Solver(...)`` builds (lbm.py:551-564, lbm.py:613-637)."""
    r = diameter / 2
    x0, y0 = 0.22 * nx, 0.5 * ny + 1.7
    geo = {"cylinder": dict(ox=x0, oy=y0, r=r),
           "sphere": dict(ox=x0, oy=y0, oz=0.5 * nz, r=r),
           "box": dict(ox=x0, oy=y0, oz=0.5 * nz, hx=r, hy=r, hz=0.3 * nz)}[obstacle]
    cfg = Config(nx, ny, nz, collision=collision, nu=u0 * diameter / reynolds, obstacle=obstacle,
                 u0=u0, sponge_start=0.75 * nx, sponge_strength=1.0, lateral=lateral, **geo)
    return replace(cfg, **extra)


# ---------------------------------------------------------------------------
# Geometry (lbm.py:144-227)

def solid(cfg, x, y, z, precision="f64"):
    """1.0 inside the obstacle, 0.0 outside, for integer or float coordinates.

    ``precision="f32"`` evaluates the same test in float32 with no fused
    multiply-add, which is how the CUDA kernels evaluate it; the tests check
    that both give the same mask for every configuration they use.
    """
    t = np.float64 if precision == "f64" else np.float32
    x, y, z = (np.asarray(a).astype(t) for a in (x, y, z))
    if cfg.obstacle == "cylinder":
        dx = x - t(cfg.ox)
        dy = y - t(cfg.oy)
        return ((dx * dx + dy * dy) < t(cfg.r) * t(cfg.r)).astype(np.float64)
    if cfg.obstacle == "sphere":
        dx = x - t(cfg.ox)
        dy = y - t(cfg.oy)
        dz = z - t(cfg.oz)
        return ((dx * dx + dy * dy + dz * dz) < t(cfg.r) * t(cfg.r)).astype(np.float64)
    if cfg.obstacle == "box":
        d = np.maximum(np.maximum(np.abs(x - t(cfg.ox)) - t(cfg.hx), np.abs(y - t(cfg.oy)) - t(cfg.hy)),
                       np.abs(z - t(cfg.oz)) - t(cfg.hz))
        return (d < 0).astype(np.float64)
    if cfg.obstacle == "heatsink":
        wall = ((y <= 0) | (y >= cfg.ny - 1)).astype(np.float64)
        return np.maximum(wall, sink(cfg, x, y, z))
    return np.zeros(np.broadcast(x, y, z).shape)


def sink(cfg, x, y, z):
    """HeatSink.sink (lbm.py:250-261): base plate and fins of the sink, 1.0 or 0.0.
    Integer coordinates; zero for every other obstacle."""
    if cfg.obstacle != "heatsink":
        return np.zeros(np.broadcast(x, y, z).shape)
    x0, length, z0, width, base, fin_h, fin_t, pitch = cfg.sink
    x1, z1 = x0 + length, z0 + width
    y_base, y_top = 1.0 + base, 1.0 + base + fin_h
    fx, fy, fz = (np.asarray(a, np.float64) for a in (x, y, z))
    inside = (fx >= x0) & (fx < x1) & (fz >= z0) & (fz < z1) & (fy >= 1.0)
    base_p = fy < y_base
    fin = (fy < y_top) & (np.mod(np.asarray(z, np.int64) - int(z0), int(pitch)) < fin_t)
    return (inside & (base_p | fin)).astype(np.float64)


def wall_velocity(cfg, xm, ym, zm):
    """Obstacle surface velocity per unit rotation rate (lbm.py:159-169, 188-198, 217-227)."""
    zero = np.zeros(np.broadcast(xm, ym, zm).shape)
    if cfg.obstacle == "cylinder" and cfg.r != 0:
        return -(ym - cfg.oy) / cfg.r, (xm - cfg.ox) / cfg.r, zero
    return zero, zero, zero


def mask(cfg, precision="f64"):
    idx = np.arange(cfg.n)
    return solid(cfg, idx % cfg.nx, (idx // cfg.nx) % cfg.ny, idx // (cfg.nx * cfg.ny), precision)


# ---------------------------------------------------------------------------
# Equilibrium and collisions (lbm.py:52-55, lbm.py:60-139)

def feq(q, rho, ux, uy, uz):
    cu = 3.0 * (float(CX[q]) * ux + float(CY[q]) * uy + float(CZ[q]) * uz)
    return W[q] * rho * (1.0 + cu + 0.5 * cu * cu - 1.5 * (ux * ux + uy * uy + uz * uz))


def smagorinsky_tau(f, rho, ux, uy, uz, tau0, cs):
    """lbm.py:72-93."""
    pxx = pyy = pzz = pxy = pxz = pyz = 0.0
    for q in range(19):
        neq = f[q] - feq(q, rho, ux, uy, uz)
        ex, ey, ez = float(CX[q]), float(CY[q]), float(CZ[q])
        pxx = pxx + ex * ex * neq
        pyy = pyy + ey * ey * neq
        pzz = pzz + ez * ez * neq
        pxy = pxy + ex * ey * neq
        pxz = pxz + ex * ez * neq
        pyz = pyz + ey * ez * neq
    pi = np.sqrt(pxx * pxx + pyy * pyy + pzz * pzz + 2.0 * (pxy * pxy + pxz * pxz + pyz * pyz))
    return 0.5 * (tau0 + np.sqrt(tau0 * tau0 + 25.456 * cs * cs * pi / rho))


def collide(cfg, f, rho, ux, uy, uz):
    """Post-collision populations and the relaxation time (lbm.py:60-139)."""
    post = np.empty_like(f)
    if cfg.collision == "bgk":
        omega = 1.0 / (3.0 * cfg.nu + 0.5)
        for q in range(19):
            post[q] = f[q] - omega * (f[q] - feq(q, rho, ux, uy, uz))
        return post, np.full(rho.shape, 1.0 / omega)
    tau0 = 3.0 * cfg.nu + 0.5
    tau = smagorinsky_tau(f, rho, ux, uy, uz, tau0, cfg.cs)
    if cfg.collision == "trt":
        omega_p = 1.0 / tau
        omega_m = 1.0 / (cfg.magic / (tau - 0.5) + 0.5)
        for q in range(19):
            o = OPP[q]
            eq = feq(q, rho, ux, uy, uz)
            eo = feq(o, rho, ux, uy, uz)
            post[q] = (f[q] - omega_p * (0.5 * (f[q] + f[o]) - 0.5 * (eq + eo))
                       - omega_m * (0.5 * (f[q] - f[o]) - 0.5 * (eq - eo)))
        return post, tau
    if cfg.collision == "les":
        omega = 1.0 / tau
        for q in range(19):
            post[q] = f[q] - omega * (f[q] - feq(q, rho, ux, uy, uz))
        return post, tau
    raise KeyError(cfg.collision)


# ---------------------------------------------------------------------------
# Kernels

def init(cfg, seed_amp=0.05):
    """lbm_init (lbm.py:383-394): equilibrium at rho = 1 with a seeded shear wave."""
    idx = np.arange(cfg.n)
    x, y, z = idx % cfg.nx, (idx // cfg.nx) % cfg.ny, idx // (cfg.nx * cfg.ny)
    fluid = 1.0 - solid(cfg, x, y, z)
    ux = cfg.u0 * fluid
    uy = (seed_amp * cfg.u0 * fluid * np.sin(6.2831853 * x.astype(float) / float(cfg.nx))
          * np.cos(6.2831853 * z.astype(float) / float(cfg.nz)))
    f = np.empty((19, cfg.n))
    for q in range(19):
        f[q] = feq(q, 1.0, ux, uy, 0.0)
    return f.reshape(-1)


def _source(cfg, q, x, y, z):
    """Where population q at (x, y, z) streams from (lbm.py:412-415, lbm.py:342-369).

    Returns the source cell, the source population, and a flag for links that
    cross the moving lid (a wall without a source cell).
    """
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    xs = (x - CX[q] + nx) % nx
    qs = np.full(x.shape, q)
    yr = y - CY[q]
    lid = np.zeros(x.shape, bool)
    if cfg.lateral == "periodic":
        ys = (yr + ny) % ny
    else:
        lo = yr < 0
        hi = yr >= ny
        out = lo | hi
        if cfg.lateral == "lid":
            lid = hi
            out = lo
        ys = np.where(out, y, np.clip(yr, 0, ny - 1))
        qs = np.where(out, MIRY[q], qs)
    zr = z - CZ[q]
    if cfg.vertical == "periodic":
        zs = (zr + nz) % nz
    else:
        out = (zr < 0) | (zr >= nz)
        zs = np.where(out, z, zr)
        qs = np.where(out, MIRZ[qs], qs)
    return xs, ys, zs, qs, lid


def step(cfg, f_in, fields=None, report=False, cells=None, dtype=np.float64):
    """One ``lbm_step`` (lbm.py:397-456, diagnostics lbm.py:493-513).

    ``f_in`` holds 19*n populations in the reference layout ``f[q*n + idx]``
    with ``idx = (z*ny + y)*nx + x``. Returns the new populations of the
    selected ``cells`` (all cells by default) as a (19, m) array. With
    ``report=True`` the 13 diagnostic fields in ``fields`` (a dict of length-n
    arrays, the previous report's values) are updated for those cells.
    """
    return _step(cfg, f_in, fields, report, cells, dtype)[0]


def step_heat(cfg, f_in, g_in, t_solid, fields=None, heat_fields=None, report=False, dtype=np.float64):
    """One ``lbm_step`` with the D3Q7 temperature block (lbm.py:457-492).

    ``g_in`` holds 7*n temperature populations ``g[q*n + idx]``, ``t_solid``
    the solid temperature per cell. Returns (f_out, g_out) as (19, n) and
    (7, n) arrays. With ``report=True`` ``heat_fields["temp"]`` is written and
    ``heat_fields["q_solid"]`` receives each fluid cell's temperature on the
    sink voxels it faces (lbm.py:484-492; the caller zeroes it first, as
    Solver.step does, lbm.py:641-642).
    """
    n = cfg.n
    out, e = _step(cfg, f_in, fields, report, None, dtype)
    G = np.asarray(g_in).reshape(7, n).astype(dtype, copy=False)
    ts = np.asarray(t_solid, dtype)
    x, y, z, idx = e["x"], e["y"], e["z"], e["idx"]
    nx, ny, nz = cfg.nx, cfg.ny, cfg.nz
    g = np.empty((7, n), dtype)
    temp = np.zeros(n, dtype)
    for q in range(7):
        o = OPP7[q]
        xs = (x - CX7[q] + nx) % nx
        ys = (y - CY7[q] + ny) % ny
        zs = (z - CZ7[q] + nz) % nz
        nidx = (zs * ny + ys) * nx + xs
        wall = solid(cfg, xs, ys, zs).astype(dtype)
        hot = sink(cfg, xs, ys, zs).astype(dtype)
        pulled = G[q, nidx]
        bounced = G[o, idx]
        at_wall = bounced * (1.0 - 2.0 * hot) + hot * 2.0 * W7[q] * ts[nidx]
        g[q] = pulled + wall * (at_wall - pulled)
        temp = temp + g[q]
    tau = e["tau"]
    alpha = cfg.alpha + np.maximum(0.0, (tau - 0.5) / 3.0 - cfg.heat_nu) / PR_T
    omega_g = 1.0 / (4.0 * alpha + 0.5)
    sigma = e["sigma"]
    temp_s = (1.0 - sigma) * temp
    ux, uy, uz = e["ux"], e["uy"], e["uz"]
    usx, usy, usz = e["ux_s"], e["uy_s"], e["uz_s"]
    g_out = np.empty_like(g)
    for q in range(7):
        eq = W7[q] * temp * (1.0 + 4.0 * (CX7[q] * ux + CY7[q] * uy + CZ7[q] * uz))
        post = g[q] - omega_g * (g[q] - eq)
        es = W7[q] * temp_s * (1.0 + 4.0 * (CX7[q] * usx + CY7[q] * usy + CZ7[q] * usz))
        g_out[q] = es + (1.0 - sigma) * (post - eq)
    if report:
        fluid, here = e["fluid"], e["here"]
        heat_fields["temp"][idx] = fluid * temp + here * ts[idx]
        for q in range(1, 7):
            xs = (x - CX7[q] + nx) % nx
            ys = (y - CY7[q] + ny) % ny
            zs = (z - CZ7[q] + nz) % nz
            nidx = (zs * ny + ys) * nx + xs
            hot = sink(cfg, xs, ys, zs)
            np.add.at(heat_fields["q_solid"], nidx, fluid * hot * temp)
    return out, g_out


def _step(cfg, f_in, fields, report, cells, dtype):
    n = cfg.n
    F = np.asarray(f_in).reshape(19, n).astype(dtype, copy=False)
    idx = np.arange(n) if cells is None else np.asarray(cells)
    nx, ny = cfg.nx, cfg.ny
    x, y, z = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    here = solid(cfg, x, y, z).astype(dtype)
    fluid = dtype(1.0) - here
    f = np.empty((19, idx.size), dtype)
    mx = np.zeros(idx.size, dtype)
    my = np.zeros(idx.size, dtype)
    mz = np.zeros(idx.size, dtype)
    omega = dtype(cfg.omega_rot)
    for q in range(19):
        o = OPP[q]
        xs, ys, zs, qs, lid = _source(cfg, q, x, y, z)
        wall = np.where(lid, 0.0, solid(cfg, xs, ys, zs)).astype(dtype)
        xm = x - 0.5 * float(CX[q])
        ym = y - 0.5 * float(CY[q])
        zm = z - 0.5 * float(CZ[q])
        vx, vy, vz = wall_velocity(cfg, xm, ym, zm)
        uw_x = np.where(lid, cfg.u_lid, omega * vx).astype(dtype)
        uw_y = np.where(lid, 0.0, omega * vy).astype(dtype)
        uw_z = np.where(lid, 0.0, omega * vz).astype(dtype)
        c_dot_uw = float(CX[q]) * uw_x + float(CY[q]) * uw_y + float(CZ[q]) * uw_z
        pulled = F[qs, (zs * ny + ys) * nx + xs]
        bounced = F[o, idx]
        bb = np.maximum(wall, lid.astype(dtype))
        w6 = dtype(6.0 * W[q])
        f[q] = pulled + bb * (bounced - pulled + w6 * c_dot_uw)
        hit = wall * fluid * (dtype(2.0) * bounced + w6 * c_dot_uw)
        mx = mx + hit * float(CX[o])
        my = my + hit * float(CY[o])
        mz = mz + hit * float(CZ[o])
    rho = np.zeros(idx.size, dtype)
    jx = np.zeros(idx.size, dtype)
    jy = np.zeros(idx.size, dtype)
    jz = np.zeros(idx.size, dtype)
    for q in range(19):
        rho = rho + f[q]
        jx = jx + f[q] * float(CX[q])
        jy = jy + f[q] * float(CY[q])
        jz = jz + f[q] * float(CZ[q])
    ux = fluid * jx / rho
    uy = fluid * jy / rho
    uz = fluid * jz / rho
    post, tau = collide(cfg, f, rho, ux, uy, uz)
    s0 = dtype(cfg.sponge_start)
    t = np.maximum(dtype(0.0), (x.astype(dtype) - s0) / (dtype(nx) - s0))
    sigma = np.maximum(here, dtype(cfg.sponge_strength) * t * t)
    rho_s = rho + sigma * (1.0 - rho)
    ux_s = ux + sigma * (dtype(cfg.u0) * fluid - ux)
    uy_s = (1.0 - sigma) * uy
    uz_s = (1.0 - sigma) * uz
    out = np.empty_like(f)
    for q in range(19):
        neq = post[q] - feq(q, rho, ux, uy, uz)
        out[q] = feq(q, rho_s, ux_s, uy_s, uz_s) + (1.0 - sigma) * neq
    if report:
        d = fields
        p = (rho - 1.0) / 3.0
        ke = 0.5 * rho * (ux * ux + uy * uy + uz * uz)
        ox, oy, oz, op = d["ux"][idx], d["uy"][idx], d["uz"][idx], d["p"][idx]
        ok = 0.5 * (ox * ox + oy * oy + oz * oz)
        d["r_rho"][idx] = (3.0 * (p - op)) * (3.0 * (p - op))
        d["r_ux"][idx] = (ux - ox) * (ux - ox)
        d["r_uy"][idx] = (uy - oy) * (uy - oy)
        d["r_uz"][idx] = (uz - oz) * (uz - oz)
        d["r_ke"][idx] = (ke - ok) * (ke - ok)
        d["ux"][idx] = ux
        d["uy"][idx] = uy
        d["uz"][idx] = uz
        d["p"][idx] = p
        d["vmag"][idx] = np.sqrt(ux * ux + uy * uy + uz * uz)
        d["fx"][idx] = mx
        d["fy"][idx] = my
        d["fz"][idx] = mz
    extras = dict(x=x, y=y, z=z, idx=idx, here=here, fluid=fluid, tau=tau, ux=ux, uy=uy, uz=uz,
                  sigma=sigma, ux_s=ux_s, uy_s=uy_s, uz_s=uz_s)
    return out, extras


def new_fields(n, dtype=np.float64):
    return {k: np.zeros(n, dtype) for k in FIELDS}


def monitors(cfg, fields, interval, diameter):
    """Solver.monitors (lbm.py:649-661) on already-computed fields."""
    n = float(cfg.n)
    total = {k: float(np.asarray(v).sum(dtype=np.float64)) for k, v in fields.items()}
    res = {name: float(np.sqrt(total[key] / n)) / max(interval, 1)
           for name, key in (("continuity", "r_rho"), ("momentum_x", "r_ux"),
                             ("momentum_y", "r_uy"), ("momentum_z", "r_uz"), ("energy", "r_ke"))}
    scale = 0.5 * cfg.u0 * cfg.u0 * diameter * cfg.nz
    res["drag"] = total["fx"] / scale
    res["lift"] = total["fy"] / scale
    return res


def run(cfg, f, steps, fields=None, report_every=0, dtype=np.float64):
    """Advance ``steps`` steps; a report step every ``report_every`` steps (0: none)."""
    f = np.asarray(f, dtype).reshape(-1)
    for k in range(steps):
        rep = report_every > 0 and (k + 1) % report_every == 0
        f = step(cfg, f, fields, report=rep, dtype=dtype).reshape(-1)
    return f


def equilibrium_state(cfg, rho, ux, uy, uz):
    """Populations at equilibrium for per-cell moments (solid cells at rest, rho = 1)."""
    fl = 1.0 - mask(cfg)
    rho = np.where(fl > 0, rho, 1.0)
    ux, uy, uz = ux * fl, uy * fl, uz * fl
    return np.concatenate([feq(q, rho, ux, uy, uz) for q in range(19)])


# ---------------------------------------------------------------------------
# Seeded start states (no reference counterpart): restatement of the CUDA
# init_random kernel, so a GPU start state can be checked independently.

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(z):
    """splitmix64 (Steele, Lea, Flood 2014) on uint64 arrays, wrapping."""
    z = np.asarray(z, np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform01(key, idx, k):
    with np.errstate(over="ignore"):
        h = splitmix64(np.uint64(key) + np.asarray(idx, np.uint64) * np.uint64(8) + np.uint64(k))
    return ((h >> np.uint64(40)).astype(np.float32) + np.float32(0.5)) * np.float32(2.0 ** -24)


def init_random(cfg, rho_sigma, u_noise, seed):
    """Equilibrium at rho = 1 + rho_sigma N(0,1), u = (u0,0,0) + U(-a,a)^3 in fluid cells."""
    key = splitmix64(np.uint64(seed))
    idx = np.arange(cfg.n)
    fl = 1.0 - mask(cfg, "f32")
    u1, u2 = uniform01(key, idx, 0), uniform01(key, idx, 1)
    g = np.sqrt(np.float32(-2.0) * np.log(u1)) * np.cos(np.float32(6.283185307179586) * u2)
    a = np.float32(u_noise)
    rho = 1.0 + fl * (np.float32(rho_sigma) * g).astype(np.float64)
    ux = fl * (cfg.u0 + (a * (np.float32(2) * uniform01(key, idx, 2) - np.float32(1))).astype(np.float64))
    uy = fl * (a * (np.float32(2) * uniform01(key, idx, 3) - np.float32(1))).astype(np.float64)
    uz = fl * (a * (np.float32(2) * uniform01(key, idx, 4) - np.float32(1))).astype(np.float64)
    return np.concatenate([feq(q, rho, ux, uy, uz) for q in range(19)])


def weight_err(a, b):
    """max |a - b| / w_q over all populations: the parity yardstick of the tests."""
    d = np.abs(np.asarray(a, np.float64).reshape(19, -1) - np.asarray(b, np.float64).reshape(19, -1))
    return float((d / W[:, None]).max())


# ---------------------------------------------------------------------------
# Derived fields on the output grid (derived.py:52-89): the velocity gradient
# by central differences, one-sided at the grid's faces, and the default
# fields |curl u| and Q = -1/2 J_ij J_ji (derived.py:27-30).

def coarsen(field, dims, stride):
    """The output grid of a field (lbm.py:516-522): every ``stride``-th cell along
    each axis, starting at 0; ceil(n / stride) points per axis."""
    nx, ny, nz = dims
    a = np.asarray(field).reshape(nz, ny, nx)
    return np.ascontiguousarray(a[::stride, ::stride, ::stride]).reshape(-1)


def velocity_gradient(ux, uy, uz, dims, inv_h):
    """(m, 3, 3) array, [p, c, d] = d u_c / d x_d at output point p."""
    mx, my, mz = dims
    u = [np.asarray(a, np.float64).reshape(mz, my, mx) for a in (ux, uy, uz)]
    out = np.zeros((mz, my, mx, 3, 3))
    for d, axis, n in ((0, 2, mx), (1, 1, my), (2, 0, mz)):
        idx = np.arange(n)
        lo, hi = np.maximum(idx - 1, 0), np.minimum(idx + 1, n - 1)
        span = (hi - lo).astype(np.float64)
        scale = np.where(span > 0, inv_h / np.where(span > 0, span, 1.0), 0.0)
        shape = [1, 1, 1]
        shape[axis] = n
        for c in range(3):
            diff = np.take(u[c], hi, axis=axis) - np.take(u[c], lo, axis=axis)
            out[..., c, d] = diff * scale.reshape(shape)
    return out.reshape(-1, 3, 3)


def vorticity_q(jac, dims, at_cells=False):
    """|curl u| and Q from a point gradient, at points or at cell centres (mean of
    the eight corner gradients)."""
    mx, my, mz = dims
    g = np.asarray(jac, np.float64).reshape(mz, my, mx, 3, 3)
    if at_cells:
        g = sum(g[k:mz - 1 + k, j:my - 1 + j, i:mx - 1 + i] for k in (0, 1) for j in (0, 1) for i in (0, 1)) / 8.0
    g = g.reshape(-1, 3, 3)
    w = np.stack([g[:, 2, 1] - g[:, 1, 2], g[:, 0, 2] - g[:, 2, 0], g[:, 1, 0] - g[:, 0, 1]], 1)
    q = -0.5 * np.einsum("pab,pba->p", g, g)
    return np.linalg.norm(w, axis=1), q
