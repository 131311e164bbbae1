"""CPU oracle for the pitch-plunge wing step (test infrastructure only).

Restates, in vectorised NumPy, tack-lbm's flutter kernels so that the CUDA
wing kernel can be checked against them; only the tests may use it.

* ``Wing.solid`` / ``wall_ux`` / ``wall_uy`` (flutter.py:20-48): a NACA 0012
  section spanning z, displaced by the plunge h and pitched by alpha about the
  elastic axis (x_ea, y_ea) at chord fraction ea; the rigid-body wall velocity.
* ``wing_init`` (flutter.py:51-58): equilibrium at rho = 1, u = (u0 fluid, 0, 0).
* ``wing_step`` (flutter.py:61-130): periodic pull streaming, halfway
  bounce-back on the moving wall, momentum exchange summed into (fx, fy, mz)
  about the displaced elastic axis, the collision, the sponge with solid cells
  relaxed to the wall velocity, and the report fields ux, uy, uz, p, vmag.
"""

from dataclasses import dataclass

import numpy as np

from oracle.lbm_oracle import CX, CY, CZ, OPP, W, collide, feq

THICK = (0.2969, -0.1260, -0.3516, 0.2843, -0.1036)  # NACA 00xx half-thickness polynomial


@dataclass
class WingConfig:
    nx: int
    ny: int
    nz: int
    chord: float
    x_ea: float
    y_ea: float
    ea: float
    state: tuple = (0.0, 0.0, 0.0, 0.0)  # h, alpha, dh/dt, dalpha/dt
    collision: str = "les"
    nu: float = 0.01
    cs: float = 0.16
    magic: float = 0.1875
    u0: float = 0.08
    sponge_start: float = 0.0
    sponge_strength: float = 1.0

    @property
    def n(self):
        return self.nx * self.ny * self.nz


def solid(c, x, y):
    """Wing.solid (flutter.py:30-42); the section is the same in every z plane."""
    h, a = c.state[0], c.state[1]
    dx = np.asarray(x, np.float64) - c.x_ea
    dy = np.asarray(y, np.float64) - (c.y_ea + h)
    s = dx * np.cos(a) - dy * np.sin(a)
    t = dx * np.sin(a) + dy * np.cos(a)
    xc = s / c.chord + c.ea
    cc = np.clip(xc, 0.0, 1.0)
    half = 0.6 * c.chord * (THICK[0] * np.sqrt(cc) + THICK[1] * cc + THICK[2] * cc ** 2 + THICK[3] * cc ** 3
                            + THICK[4] * cc ** 4)
    return ((xc >= 0.0) & (xc <= 1.0) & (np.abs(t) < half)).astype(np.float64)


def wall_u(c, x, y):
    """Rigid-body velocity of the wing at (x, y) (flutter.py:44-50)."""
    h, _, dh, da = c.state
    return da * (y - c.y_ea - h), dh - da * (x - c.x_ea)


def init(c):
    idx = np.arange(c.n)
    x, y = idx % c.nx, (idx // c.nx) % c.ny
    ux = c.u0 * (1.0 - solid(c, x, y))
    return np.concatenate([feq(q, 1.0, ux, 0.0, 0.0) for q in range(19)])


def step(c, f_in, fields=None, report=False):
    """One wing_step: returns (f_out (19, n), (fx, fy, mz))."""
    n = c.n
    F = np.asarray(f_in, np.float64).reshape(19, n)
    idx = np.arange(n)
    x, y, z = idx % c.nx, (idx // c.nx) % c.ny, idx // (c.nx * c.ny)
    here = solid(c, x, y)
    fluid = 1.0 - here
    f = np.empty((19, n))
    fx = np.zeros(n)
    fy = np.zeros(n)
    mz = np.zeros(n)
    for q in range(19):
        o = OPP[q]
        xs = (x - CX[q]) % c.nx
        ys = (y - CY[q]) % c.ny
        zs = (z - CZ[q]) % c.nz
        wall = solid(c, xs, ys)
        pulled = F[q, (zs * c.ny + ys) * c.nx + xs]
        bounced = F[o, idx]
        px = x - 0.5 * CX[q]
        py = y - 0.5 * CY[q]
        wx, wy = wall_u(c, px, py)
        back = bounced + 6.0 * W[q] * (CX[q] * wx + CY[q] * wy)
        f[q] = pulled + wall * (back - pulled)
        hit = wall * fluid * (bounced + back)
        dfx, dfy = hit * CX[o], hit * CY[o]
        fx += dfx
        fy += dfy
        mz += (px - c.x_ea) * dfy - (py - c.y_ea - c.state[0]) * dfx
    rho = f.sum(0)
    ux = fluid * (CX[:, None] * f).sum(0) / rho
    uy = fluid * (CY[:, None] * f).sum(0) / rho
    uz = fluid * (CZ[:, None] * f).sum(0) / rho
    post, _ = collide(c, f, rho, ux, uy, uz)
    t = np.maximum(0.0, (x - c.sponge_start) / (c.nx - c.sponge_start))
    sigma = np.maximum(here, c.sponge_strength * t * t)
    wx, wy = wall_u(c, x.astype(np.float64), y.astype(np.float64))
    tx = fluid * c.u0 + here * wx
    ty = here * wy
    rho_s = rho + sigma * (1.0 - rho)
    ux_s = ux + sigma * (tx - ux)
    uy_s = uy + sigma * (ty - uy)
    uz_s = (1.0 - sigma) * uz
    out = np.empty_like(f)
    for q in range(19):
        out[q] = feq(q, rho_s, ux_s, uy_s, uz_s) + (1.0 - sigma) * (post[q] - feq(q, rho, ux, uy, uz))
    if report:
        fields["ux"][:], fields["uy"][:], fields["uz"][:] = ux, uy, uz
        fields["p"][:] = (rho - 1.0) / 3.0
        fields["vmag"][:] = np.sqrt(ux * ux + uy * uy + uz * uz)
    return out, (float(fx.sum()), float(fy.sum()), float(mz.sum()))
