"""CPU oracle for the cantilever-wing FSI step (test infrastructure only).

Restates tack-lbm's fsi kernels in NumPy so the CUDA FSI kernel can be checked
against them; only the tests may use it.

* ``FlexWing.solid`` (fsi.py:35-47): the NACA 0012 section of layer z, with
  that layer's plunge h and pitch alpha, for z + 1/2 < span.
* ``FlexWing.wall_fraction`` (fsi.py:49-60): where the wall cuts a link, by six
  bisection steps on the section test (the layer switches to the source
  layer past the link's midpoint).
* ``fsi_init`` (fsi.py:71-78) and ``fsi_step`` (fsi.py:81-186): inflow at
  x = 0 (the free-stream equilibrium), zero-gradient outflow at x = nx - 1,
  periodic y, mirror (free-slip) planes below z = 0 and above z = nz - 1,
  moving-wall bounce-back made second order by the interpolated (Bouzidi)
  rule on wetted links, the momentum exchange relative to the fluid at rest
  summed per layer, the collision, the sponge (density and
  non-equilibrium only; solid cells take the wall velocity), report fields.
"""

from dataclasses import dataclass

import numpy as np

from oracle.lbm_oracle import CX, CY, CZ, MIRZ, OPP, W, collide, feq
from oracle.flutter_oracle import THICK


@dataclass
class FsiConfig:
    nx: int
    ny: int
    nz: int
    chord: float
    x_ea: float
    y_ea: float
    ea: float
    span: float
    kin: np.ndarray = None  # (nz, 4): h, alpha, dh/dt, dalpha/dt per layer
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


def solid(c, x, y, z):
    """FlexWing.solid for float x, y and integer layer z (arrays broadcast)."""
    z = np.asarray(z, np.int64)
    h, a = c.kin[z, 0], c.kin[z, 1]
    dx = np.asarray(x, np.float64) - c.x_ea
    dy = np.asarray(y, np.float64) - (c.y_ea + h)
    s = dx * np.cos(a) - dy * np.sin(a)
    t = dx * np.sin(a) + dy * np.cos(a)
    xc = s / c.chord + c.ea
    cc = np.clip(xc, 0.0, 1.0)
    half = 0.6 * c.chord * (THICK[0] * np.sqrt(cc) + THICK[1] * cc + THICK[2] * cc ** 2 + THICK[3] * cc ** 3
                            + THICK[4] * cc ** 4)
    inside = (xc >= 0.0) & (xc <= 1.0) & (np.abs(t) < half)
    return (inside & (z + 0.5 < c.span)).astype(np.float64)


def wall_fraction(c, x, y, z, cx, cy, zs):
    lo = np.zeros(np.broadcast(x, y, z).shape)
    hi = np.ones_like(lo)
    for _ in range(6):
        mid = 0.5 * (lo + hi)
        zl = np.where(mid >= 0.5, zs, z)
        inside = solid(c, x - mid * cx, y - mid * cy, zl)
        hi = hi + inside * (mid - hi)
        lo = lo + (1.0 - inside) * (mid - lo)
    return 0.5 * (lo + hi)


def wall_u(c, x, y, z):
    k = c.kin[np.asarray(z, np.int64)]
    return k[..., 3] * (y - c.y_ea - k[..., 0]), k[..., 2] - k[..., 3] * (x - c.x_ea)


def init(c):
    idx = np.arange(c.n)
    x, y, z = idx % c.nx, (idx // c.nx) % c.ny, idx // (c.nx * c.ny)
    ux = c.u0 * (1.0 - solid(c, x, y, z))
    return np.concatenate([feq(q, 1.0, ux, 0.0, 0.0) for q in range(19)])


def step(c, f_in, fields=None, report=False):
    """One fsi_step: returns (f_out (19, n), load (nz, 3) = per-layer fx, fy, mz)."""
    n, nx, ny, nz = c.n, c.nx, c.ny, c.nz
    F = np.asarray(f_in, np.float64).reshape(19, n)
    idx = np.arange(n)
    x, y, z = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    here = solid(c, x, y, z)
    fluid = 1.0 - here
    f = np.empty((19, n))
    fx, fy, mz = np.zeros(n), np.zeros(n), np.zeros(n)
    for q in range(19):
        o = OPP[q]
        xr = x - CX[q]
        xs = np.clip(xr, 0, nx - 1)
        inflow = xr < 0
        ys = (y - CY[q]) % ny
        zr = z - CZ[q]
        flip = (zr < 0) | (zr > nz - 1)
        zs = np.clip(zr, 0, nz - 1)
        qs = np.where(flip, MIRZ[q], q)
        wall = solid(c, xs, ys, zs)
        pulled = F[qs, (zs * ny + ys) * nx + xs]
        pulled = np.where(inflow, feq(q, 1.0, c.u0, 0.0, 0.0), pulled)
        bounced = F[o, idx]
        px = x - 0.5 * CX[q]
        py = y - 0.5 * CY[q]
        wx, wy = wall_u(c, px, py, zs)
        back = bounced + 6.0 * W[q] * (CX[q] * wx + CY[q] * wy)
        wet = wall * fluid > 0.5
        if wet.any():
            i = np.flatnonzero(wet)
            xi, yi, zi, zsi = x[i], y[i], z[i], zs[i]
            delta = wall_fraction(c, xi.astype(np.float64), yi.astype(np.float64), zi, CX[q], CY[q], zsi)
            pxi = xi - delta * CX[q]
            pyi = yi - delta * CY[q]
            wxi, wyi = wall_u(c, pxi, pyi, zsi)
            cui = CX[q] * wxi + CY[q] * wyi
            far = delta >= 0.5
            b_far = (bounced[i] + (2.0 * delta - 1.0) * F[q, i] + 6.0 * W[q] * cui) / (2.0 * delta)
            xn = (xi + CX[q]) % nx
            yn = (yi + CY[q]) % ny
            zn = zi + CZ[q]
            zc = np.clip(zn, 0, nz - 1)
            open_behind = (zn == zc) * (1.0 - solid(c, xn, yn, zc))
            behind = F[o, (zc * ny + yn) * nx + xn]
            ibb = 2.0 * delta * bounced[i] + (1.0 - 2.0 * delta) * behind + 6.0 * W[q] * cui
            b_near = back[i] + open_behind * (ibb - back[i])
            back[i] = np.where(far, b_far, b_near)
            px = px.astype(np.float64)
            py = py.astype(np.float64)
            px[i], py[i] = pxi, pyi
        f[q] = pulled + wall * (back - pulled)
        hit = wall * fluid * (bounced + back - 2.0 * W[q])
        dfx, dfy = hit * CX[o], hit * CY[o]
        fx += dfx
        fy += dfy
        mz += (px - c.x_ea) * dfy - (py - c.y_ea - c.kin[z, 0]) * dfx
    load = np.zeros((nz, 3))
    for k, v in enumerate((fx, fy, mz)):
        np.add.at(load[:, k], z, v)
    rho = f.sum(0)
    ux = fluid * (CX[:, None] * f).sum(0) / rho
    uy = fluid * (CY[:, None] * f).sum(0) / rho
    uz = fluid * (CZ[:, None] * f).sum(0) / rho
    post, _ = collide(c, f, rho, ux, uy, uz)
    t = np.maximum(0.0, (x - c.sponge_start) / (nx - c.sponge_start))
    sigma = np.maximum(here, c.sponge_strength * t * t)
    wx, wy = wall_u(c, x.astype(np.float64), y.astype(np.float64), z)
    rho_s = rho + sigma * (1.0 - rho)
    ux_s = ux + here * (wx - ux)
    uy_s = uy + here * (wy - uy)
    uz_s = (1.0 - here) * uz
    out = np.empty_like(f)
    for q in range(19):
        out[q] = feq(q, rho_s, ux_s, uy_s, uz_s) + (1.0 - sigma) * (post[q] - feq(q, rho, ux, uy, uz))
    if report:
        fields["ux"][:], fields["uy"][:], fields["uz"][:] = ux, uy, uz
        fields["p"][:] = (rho - 1.0) / 3.0
        fields["vmag"][:] = np.sqrt(ux * ux + uy * uy + uz * uz)
    return out, load
