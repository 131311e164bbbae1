"""The FSI kernel's block-level wing test (block_near_wing in
tack-lbm_gb300/csrc/lbm_fsi.cu), restated in float32 NumPy, never skips a
block that can pull from a wing cell (CPU).

A 32 x 4-cell block of layer z skips every mask load when the squares of
1.01 chord + 1 around the displaced elastic axes of layers z-1..z+1 miss its
sources [x0-1, x0+32] x [y0-1, y0+4]; blocks on the periodic y edges are
always checked. The test takes FSISolver's default lattice (256 x 128 x 104,
chord 32, span 64) with large plunge and twist, computes the oracle's float64
section mask (fsi.py:35-47) over the whole lattice, and checks that no
skipped block has a solid cell among its sources."""

import numpy as np

from oracle import fsi_oracle as FS

F = np.float32
BX, BY = 32, 4


def _naca_f(c):
    """Per-layer prefilter inputs as the host builds them (lbm_naca.cuh make_naca_f)."""
    xc0 = np.full(c.nz, F(c.x_ea))
    yc0 = (c.y_ea + c.kin[:, 0]).astype(F)
    reach = np.full(c.nz, F(1.01 * c.chord + 1.0))
    reach[~(np.arange(c.nz) + 0.5 < c.span)] = F(-1.0)
    return xc0, yc0, reach


def _near(c, xb, yb, z):
    if yb == 0 or yb + BY >= c.ny:
        return True
    xc0, yc0, reach = _naca_f(c)
    x0, x1, y0, y1 = F(xb - 1), F(xb + BX), F(yb - 1), F(yb + BY)
    for zz in range(max(z - 1, 0), min(z + 1, c.nz - 1) + 1):
        r = reach[zz]
        if r >= 0 and x1 >= xc0[zz] - r and x0 <= xc0[zz] + r and y1 >= yc0[zz] - r and y0 <= yc0[zz] + r:
            return True
    return False


def test_skipped_blocks_see_no_wing():
    nx, ny, nz = 256, 128, 104
    rng = np.random.default_rng(3)
    for trial in range(3):
        zs = np.arange(nz) + 0.5
        s = np.clip(zs / 64.0, 0, None)
        kin = np.zeros((nz, 4))
        kin[:, 0] = rng.uniform(-12, 12) * s ** 2          # plunge up to ~0.4 chord at the tip
        kin[:, 1] = np.radians(rng.uniform(-15, 15)) * s   # twist up to 15 degrees
        c = FS.FsiConfig(nx, ny, nz, 32.0, 0.25 * nx, 0.5 * ny, 0.4, 64.0, kin=kin)
        idx = np.arange(c.n)
        x, y, z = idx % nx, (idx // nx) % ny, idx // (nx * ny)
        solid = FS.solid(c, x, y, z).reshape(nz, ny, nx) > 0
        assert solid.any()
        # solid anywhere in each cell's source box: dilate by one cell in x, y (periodic), z
        d = solid.copy()
        d[:, :, 1:] |= solid[:, :, :-1]
        d[:, :, :-1] |= solid[:, :, 1:]
        e = d | np.roll(d, 1, axis=1) | np.roll(d, -1, axis=1)
        g = e.copy()
        g[1:] |= e[:-1]
        g[:-1] |= e[1:]
        # per block of BX x BY cells of one layer
        blocks = g.reshape(nz, ny // BY, BY, nx // BX, BX).any(axis=(2, 4))
        skipped = wing = 0
        for zz in range(nz):
            for by in range(ny // BY):
                for bx in range(nx // BX):
                    if not _near(c, bx * BX, by * BY, zz):
                        skipped += 1
                        assert not blocks[zz, by, bx], (trial, zz, by, bx)
                    elif blocks[zz, by, bx]:
                        wing += 1
        assert wing > 0 and skipped > 0.7 * blocks.size  # ~76 % of blocks skip the mask loads
