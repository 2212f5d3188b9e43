"""numpy restatement of the FP64 diagnostics (test infrastructure only).

Node charge density (trilinear weights, node (i,j,k) at the low corner of
voxel (i,j,k), periodic fold of the n+1 node layer), the discrete Gauss
residual div E - rho/eps0 with backward differences of the edge fields and
periodic images for index 0, and kinetic energy sum w m c^2 (gamma - 1).
The reference has no such diagnostics; these are the quantities its push
and Yee update conserve (checked by tests/test_diagnostics_gpu.py)."""
from __future__ import annotations

import numpy as np


def _rank_to_index(c, nx, ny):
    sx, sy = nx + 2, ny + 2
    iy, ix = np.divmod(c, sx)
    iz, iy = np.divmod(iy, sy)
    return ix, iy, iz


def charge_density(p, nx, ny, nz, qsp, dx, dy, dz):
    """p: dict of particle arrays; returns rho as (nz+2, ny+2, nx+2) float64."""
    sx, sy, sz = nx + 2, ny + 2, nz + 2
    rho = np.zeros(sx * sy * sz)
    c = p["cell"].astype(np.int64)
    x, y, z = (p[k].astype(np.float64) for k in ("x", "y", "z"))
    q = p["w"].astype(np.float64) * (qsp / (dx * dy * dz))
    wx = (0.5 * (1 - x), 0.5 * (1 + x))
    wy = (0.5 * (1 - y), 0.5 * (1 + y))
    wz = (0.5 * (1 - z), 0.5 * (1 + z))
    for a in (0, 1):
        for b in (0, 1):
            for d in (0, 1):
                np.add.at(rho, c + a + sx * b + sx * sy * d, q * wx[a] * wy[b] * wz[d])
    r = rho.reshape(sz, sy, sx)
    r[:, :, 1] += r[:, :, nx + 1]; r[:, :, nx + 1] = 0
    r[:, 1, :] += r[:, ny + 1, :]; r[:, ny + 1, :] = 0
    r[1, :, :] += r[nz + 1, :, :]; r[nz + 1, :, :] = 0
    return r


def div_e(fields_cells, nx, ny, nz, dx, dy, dz):
    """fields_cells: (num_cells, 9) member array; returns div E at interior
    nodes as (nz, ny, nx) float64."""
    F = fields_cells.astype(np.float64).reshape(nz + 2, ny + 2, nx + 2, 9)
    e = [F[..., m].copy() for m in range(3)]
    for a in e:  # periodic images of the index-0 layer
        a[:, :, 0] = a[:, :, nx]
        a[:, 0, :] = a[:, ny, :]
        a[0, :, :] = a[nz, :, :]
    ex, ey, ez = e
    I = np.s_[1:nz + 1, 1:ny + 1, 1:nx + 1]
    return ((ex[I] - ex[1:nz + 1, 1:ny + 1, 0:nx]) / dx
            + (ey[I] - ey[1:nz + 1, 0:ny, 1:nx + 1]) / dy
            + (ez[I] - ez[0:nz, 1:ny + 1, 1:nx + 1]) / dz)


def gauss_residual(fields_cells, rho, nx, ny, nz, dx, dy, dz, eps0=1.0):
    return div_e(fields_cells, nx, ny, nz, dx, dy, dz) - rho[1:nz + 1, 1:ny + 1, 1:nx + 1] / eps0


def kinetic_energy(p, mc2=1.0):
    u2 = sum(p[k].astype(np.float64) ** 2 for k in ("ux", "uy", "uz"))
    return mc2 * float(np.sum(p["w"].astype(np.float64) * (u2 / (1 + np.sqrt(1 + u2)))))
