"""Pure-PyTorch FP64 reference of the differentiable drag model (test infrastructure only).

The checker for the native adjoint (``lbm_adj_*``): the same smoothed-cylinder
LES step, written with torch tensor operations so that ``torch.autograd``
gives the reference gradient of the loss with respect to (U, tau0, Cs, r).
Only the tests may use it; the product path never does.

Model (restating tack-lbm's step, lbm.py:397-456, with the 0/1 solid test
replaced by phi = (1 + tanh((r - d)/width))/2, d the distance to the
cylinder axis):

* start state: f = feq(1, (U fl, A U fl sin(2 pi x/nx) cos(2 pi z/nz), 0)),
  fl = 1 - phi (lbm_init, lbm.py:383-394);
* streaming: p_q = f_q(x - c_q), b_q = f_{opp q}(x),
  g_q = p_q + phi(x - c_q)(b_q - p_q) (lbm.py:410-428; periodic);
* momentum exchange: F_x = sum_q phi(x - c_q) fl 2 b_q c_{opp q, x} (lbm.py:429-432);
* moments rho = sum g, u = fl j / rho (lbm.py:433-439);
* LES: tau = (tau0 + sqrt(tau0^2 + 25.456 Cs^2 |Pi| / rho))/2, Pi the
  non-equilibrium second moment of g (lbm.py:72-93, 126-139), post = g + (feq - g)/tau;
* sponge: sigma = 1 - fl (1 - S t^2), t = max(0, (x - s0)/(nx - s0));
  rho_s = rho + sigma (1 - rho), u_s = (u_x + sigma (U fl - u_x), (1 - sigma) u_y,
  (1 - sigma) u_z); out = feq(rho_s, u_s) + (1 - sigma)(post - feq(rho, u)) (lbm.py:446-456).

The loss is sum_{t >= loss_start} F_x(t) / (N_l 0.5 U^2 D nz), F_x(t) computed by
step t from the state before it. Weights are the float32-rounded D3Q19 weights
the reference uploads (lbm.py:18, lbm.py:48).
"""

import numpy as np
import torch
from torch.utils.checkpoint import checkpoint as _checkpoint

from oracle.lbm_oracle import CX as _CX, CY as _CY, CZ as _CZ, OPP as _OPP, W

CX, CY, CZ, OPP = (list(map(int, a)) for a in (_CX, _CY, _CZ, _OPP))
SMAG = 25.456


class Model:
    """Geometry and schedule of one run (lengths in lattice cells)."""

    def __init__(self, nx, ny, nz, *, steps, loss_start, ox, oy, width, diameter, sponge_start,
                 sponge_strength=1.0, seed_amp=0.05):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.steps, self.loss_start = steps, loss_start
        self.ox, self.oy, self.width, self.diameter = ox, oy, width, diameter
        self.sponge_start, self.sponge_strength, self.seed_amp = sponge_start, sponge_strength, seed_amp
        dt = torch.float64
        z, y, x = torch.meshgrid(torch.arange(nz, dtype=dt), torch.arange(ny, dtype=dt),
                                 torch.arange(nx, dtype=dt), indexing="ij")
        self.x, self.z = x, z
        self.d = torch.sqrt((x - ox) ** 2 + (y - oy) ** 2)
        t = torch.clamp((x - sponge_start) * (1.0 / (nx - sponge_start)), min=0.0)
        self.sp = sponge_strength * t * t
        self.wave = seed_amp * torch.sin(2 * np.pi * x / nx) * torch.cos(2 * np.pi * z / nz)
        self.w = torch.tensor(W, dtype=dt).view(19, 1, 1, 1)
        self.cx = torch.tensor(CX, dtype=dt).view(19, 1, 1, 1)
        self.cy = torch.tensor(CY, dtype=dt).view(19, 1, 1, 1)
        self.cz = torch.tensor(CZ, dtype=dt).view(19, 1, 1, 1)


def feq(m, rho, ux, uy, uz):
    s = m.cx * ux + m.cy * uy + m.cz * uz
    usq = ux * ux + uy * uy + uz * uz
    return m.w * rho * (1 + 3 * s + 4.5 * s * s - 1.5 * usq)


def shifted(a, q):
    """a(x - c_q) with periodic wrap."""
    return torch.roll(a, shifts=(CZ[q], CY[q], CX[q]), dims=(-3, -2, -1))


def start_state(m, u0, phi):
    fl = 1 - phi
    ux = u0 * fl
    uy = m.wave * u0 * fl
    return feq(m, torch.ones_like(phi), ux, uy, torch.zeros_like(phi))


def step(m, f, u0, tau0, cs, phi):
    """One step; returns (f_next, F_x summed over the lattice)."""
    fl = 1 - phi
    g, force = [f[0]], 0.0
    for q in range(1, 19):
        ps = shifted(phi, q)
        p = shifted(f[q], q)
        b = f[OPP[q]]
        g.append(p + ps * (b - p))
        if CX[q]:
            force = force + (-CX[q]) * (ps * fl * 2 * b).sum()
    g = torch.stack(g)
    rho = g.sum(0)
    jx, jy, jz = (m.cx * g).sum(0), (m.cy * g).sum(0), (m.cz * g).sum(0)
    ux, uy, uz = fl * jx / rho, fl * jy / rho, fl * jz / rho
    e0 = feq(m, rho, ux, uy, uz)
    ne = g - e0
    pxx, pyy, pzz = (m.cx * m.cx * ne).sum(0), (m.cy * m.cy * ne).sum(0), (m.cz * m.cz * ne).sum(0)
    pxy, pxz, pyz = (m.cx * m.cy * ne).sum(0), (m.cx * m.cz * ne).sum(0), (m.cy * m.cz * ne).sum(0)
    pn = torch.sqrt(pxx ** 2 + pyy ** 2 + pzz ** 2 + 2 * (pxy ** 2 + pxz ** 2 + pyz ** 2))
    tau = 0.5 * (tau0 + torch.sqrt(tau0 * tau0 + SMAG * cs * cs * pn / rho))
    post = g + (e0 - g) / tau
    sigma = 1 - fl * (1 - m.sp)
    keep = 1 - sigma
    rhos = rho + sigma * (1 - rho)
    usx = ux + sigma * (u0 * fl - ux)
    e1 = feq(m, rhos, usx, keep * uy, keep * uz)
    return e1 + keep * (post - e0), force


def loss(m, params, segment=10):
    """The drag loss at params = (U, tau0, Cs, r) (a float64 4-tensor);
    autograd-differentiable. Steps run in checkpointed segments."""
    u0, tau0, cs, r = params[0], params[1], params[2], params[3]
    phi = 0.5 * (1 + torch.tanh((r - m.d) / m.width))
    f = start_state(m, u0, phi)
    total = torch.zeros((), dtype=torch.float64)

    def run(f, t0, t1):
        acc = torch.zeros((), dtype=torch.float64)
        for t in range(t0, t1):
            f, force = step(m, f, u0, tau0, cs, phi)
            if t >= m.loss_start:
                acc = acc + force
        return f, acc

    t = 1
    while t <= m.steps:
        t1 = min(t + segment, m.steps + 1)
        f, acc = _checkpoint(run, f, t, t1, use_reentrant=False)
        total = total + acc
        t = t1
    nl = m.steps - m.loss_start + 1
    return total / (nl * 0.5 * u0 * u0 * m.diameter * m.nz)


def gradient(m, params):
    """(loss, dloss/dparams) as float64 numpy values."""
    p = torch.tensor(np.asarray(params, np.float64), dtype=torch.float64, requires_grad=True)
    value = loss(m, p)
    value.backward()
    return float(value.detach()), p.grad.numpy().copy()


def central_differences(m, params, rel=1e-4):
    """Central differences of the loss, step rel*|p_k| per parameter."""
    p0 = np.asarray(params, np.float64)
    out = np.zeros(4)
    with torch.no_grad():
        for k in range(4):
            h = rel * abs(p0[k])
            hi, lo = p0.copy(), p0.copy()
            hi[k] += h
            lo[k] -= h
            out[k] = (float(loss(m, torch.tensor(hi))) - float(loss(m, torch.tensor(lo)))) / (2 * h)
    return out
