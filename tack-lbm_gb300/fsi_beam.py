"""Cantilever wing beam for the FSI solver: 1-D finite elements along the span.

tack-lbm's default structural model (fsi_beam.py:29-126 there) assembles a
Timoshenko bending beam and a St. Venant torsion bar on the elastic axis with
MFEM, couples them through the section's mass (its centre of gravity sits
behind the elastic axis) and keeps the lowest modes. MFEM is not needed for
that: the model is one-dimensional. This module assembles the same bilinear
forms with its own H1 Lagrange elements (Gauss-Lobatto nodes, exact Gauss
quadrature) and solves the same generalised eigenproblem with SciPy.

Per unit span, fluid density 1, semichord b:
    m = mu pi b^2, S_alpha = m x_alpha b, I_alpha = m r_alpha2 b^2, GJ = 1,
    EI from the uncoupled cantilever frequency ratio freq_ratio =
    omega_bend / omega_twist = (1.875^2 sqrt(EI / m L^4)) / ((pi/2) sqrt(GJ / I_alpha L^2)),
    kGA = 1000 EI / h_e^2 (a shear-stiff Timoshenko beam).
Unknowns (w, theta, phi): deflection, bending rotation and twist, all clamped
at the root z = 0. Stiffness
    [[kGA K1, -kGA D^T, 0], [-kGA D, EI K1 + kGA M1, 0], [0, 0, GJ K1]]
and mass
    [[m M1, 0, -S_alpha M1], [0, m (0.05 c)^2 M1, 0], [-S_alpha M1, 0, I_alpha M1]]
with K1 = (N_i', N_j'), M1 = (N_i, N_j), D = (N_i, N_j') (fsi_beam.py:50-79).
A section at span station z moves by the plunge of the reference axis,
h = w + (elastic_axis - ea) c phi, and the pitch alpha = phi (fsi_beam.py:95-101).
"""

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as sla
from numpy.polynomial import legendre


def naca_half(xc):
    """NACA 0012 half thickness over the chord, xc in [0, 1] (fsi_struct.py:19-21)."""
    xc = np.clip(xc, 0.0, 1.0)
    return 0.6 * (0.2969 * np.sqrt(xc) - 0.126 * xc - 0.3516 * xc ** 2 + 0.2843 * xc ** 3 - 0.1036 * xc ** 4)


def _element(order):
    """Reference element on [0, 1]: Gauss-Lobatto nodes and the three local
    matrices (N_a', N_b'), (N_a, N_b), (N_a, N_b') for unit length."""
    if order < 1:
        raise ValueError("order must be >= 1")
    inner = legendre.Legendre.basis(order).deriv().roots() if order > 1 else np.zeros(0)
    nodes = 0.5 * (np.concatenate([[-1.0], np.sort(inner.real), [1.0]]) + 1.0)
    # Lagrange basis through the nodes: coefficients by inverting the Vandermonde matrix
    coef = np.linalg.inv(np.vander(nodes, order + 1, increasing=True))  # column a: basis a
    xq, wq = legendre.leggauss(order + 2)
    xq, wq = 0.5 * (xq + 1.0), 0.5 * wq
    powers = np.vander(xq, order + 1, increasing=True)
    dpowers = np.zeros_like(powers)
    dpowers[:, 1:] = powers[:, :-1] * np.arange(1, order + 1)
    n, dn = powers @ coef, dpowers @ coef  # (quad point, basis)
    stiff = (dn * wq[:, None]).T @ dn
    mass = (n * wq[:, None]).T @ n
    mixed = (n * wq[:, None]).T @ dn  # row a: test N_a, column b: trial N_b'
    return nodes, stiff, mass, mixed


def assemble(span, elements, order):
    """Global K1, M1, D (CSR) and the dof positions, numbered from the root out."""
    nodes, ks, ms, ds = _element(order)
    le = span / elements
    size = elements * order + 1
    rows, cols, kv, mv, dv = [], [], [], [], []
    for e in range(elements):
        g = e * order + np.arange(order + 1)
        r, c = np.meshgrid(g, g, indexing="ij")
        rows.append(r.ravel())
        cols.append(c.ravel())
        kv.append((ks / le).ravel())
        mv.append((ms * le).ravel())
        dv.append(ds.ravel())
    rows, cols = np.concatenate(rows), np.concatenate(cols)

    def csr(v):
        return sp.csr_matrix((np.concatenate(v), (rows, cols)), shape=(size, size))

    z = np.empty(size)
    for e in range(elements):
        z[e * order:e * order + order + 1] = (e + nodes) * le
    return csr(kv), csr(mv), csr(dv), z


class WingBeam:
    """The reference's WingBeam (same arguments and attributes: ``omega0``,
    ``h``, ``alpha``, ``layer_z``, ``sections_at``, ``quads``, ``rest``,
    ``deformed``), assembled without MFEM."""

    def __init__(self, chord=32.0, span=64.0, ea=0.4, elastic_axis=0.15, mu=8.0, x_alpha=0.4, r_alpha2=0.5,
                 freq_ratio=0.6, elements=32, order=2, modes=6, sections=33, contour=40):
        self.chord, self.span, self.ea = chord, span, ea
        self.elastic_axis, self.mu, self.x_alpha, self.r_alpha2 = elastic_axis, mu, x_alpha, r_alpha2
        b = 0.5 * chord
        m = mu * np.pi * b * b
        s_alpha = m * x_alpha * b
        i_alpha = m * r_alpha2 * b * b
        gj = 1.0
        ei = m * (gj / i_alpha) * (freq_ratio * np.pi * span / (2.0 * 1.875 ** 2)) ** 2
        kga = 1.0e3 * ei / (span / elements) ** 2
        k1, m1, d, z = assemble(span, elements, order)
        n = z.size
        zero = sp.csr_matrix((n, n))
        stiffness = sp.bmat([[kga * k1, -kga * d.T, zero],
                             [-kga * d, ei * k1 + kga * m1, zero],
                             [zero, zero, gj * k1]]).tocsc()
        mass = sp.bmat([[m * m1, zero, -s_alpha * m1],
                        [zero, m * (0.05 * chord) ** 2 * m1, zero],
                        [-s_alpha * m1, zero, i_alpha * m1]]).tocsc()
        free = np.setdiff1d(np.arange(3 * n), [0, n, 2 * n])  # clamped root: w, theta, phi at z = 0
        kf, mf = stiffness[free][:, free], mass[free][:, free]
        w2, vec = sla.eigsh(kf, k=modes, M=mf, sigma=0.0, which="LM", v0=np.ones(free.size))
        order_ = np.argsort(w2)
        self.omega0 = np.sqrt(np.maximum(w2[order_], 0.0))
        shapes = np.zeros((modes, 3 * n))
        shapes[:, free] = vec[:, order_].T
        w, twist = shapes[:, :n], shapes[:, 2 * n:]
        # a fixed sign: each mode's dominant tip motion (plunge or semichord x twist) is positive
        tip = np.where(np.abs(w[:, -1]) >= b * np.abs(twist[:, -1]), w[:, -1], twist[:, -1])
        sign = np.where(tip < 0.0, -1.0, 1.0)[:, None]
        w, twist = w * sign, twist * sign
        self.layer_z = z
        self.h = w + twist * (elastic_axis - ea) * chord
        self.alpha = twist
        self._surface(sections, contour)

    def sections_at(self, zs):
        """Modal plunge and pitch (modes x stations) at span stations zs; zero beyond the tip."""
        zs = np.asarray(zs, float)
        inside = zs <= self.span
        h = np.array([np.interp(zs, self.layer_z, row) * inside for row in self.h])
        a = np.array([np.interp(zs, self.layer_z, row) * inside for row in self.alpha])
        return h, a

    def _surface(self, sections, contour):
        """A quad mesh of the wing surface: ``contour`` points per side on
        ``sections`` stations, closed at the trailing edge and the tip,
        normals pointing out."""
        beta = np.linspace(0.0, np.pi, contour)
        xc = 0.5 * (1.0 - np.cos(beta))
        half = naca_half(xc)
        self._ring = ((np.concatenate([xc, xc]) - self.ea) * self.chord,
                      np.concatenate([half, -half]) * self.chord)
        self._stations = np.linspace(0.0, self.span, sections)
        k = contour
        ring = 2 * k
        faces = []
        for s in range(sections - 1):
            lo, hi = s * ring, (s + 1) * ring
            j = np.arange(k - 1)
            faces.append(np.stack([lo + j, lo + j + 1, hi + j + 1, hi + j], 1))              # upper side
            faces.append(np.stack([lo + k + j + 1, lo + k + j, hi + k + j, hi + k + j + 1], 1))  # lower side
            faces.append(np.array([[lo + k - 1, lo + ring - 1, hi + ring - 1, hi + k - 1]]))  # trailing edge
        top = (sections - 1) * ring
        j = np.arange(k - 1)
        faces.append(np.stack([top + j, top + j + 1, top + k + j + 1, top + k + j], 1))      # tip cap
        self.quads = np.concatenate(faces).astype(np.int64)[:, ::-1].copy()
        self.rest = self.deformed(np.zeros(len(self.omega0)))

    def deformed(self, q):
        """Surface points (stations x ring, 3) at modal amplitudes q."""
        hm, am = self.sections_at(self._stations)
        h, a = q @ hm, q @ am
        s, t = self._ring
        ca, sa = np.cos(a)[:, None], np.sin(a)[:, None]
        x = s[None, :] * ca + t[None, :] * sa
        y = h[:, None] - s[None, :] * sa + t[None, :] * ca
        zz = np.broadcast_to(self._stations[:, None], x.shape)
        return np.stack([x, y, zz], -1).reshape(-1, 3)
