"""Host-side packing of the reference's array layouts (include/cpic/layout.h).

particle_list_t   AoSoA<real_t x7, int>, vector length vl: per SoA block
                  x[vl] y[vl] z[vl] ux[vl] uy[vl] uz[vl] w[vl] cell[vl]
interpolator/field AoSoA with 32-cell blocks, 18 / 9 members
accumulator       [num_cells][3][4] (LayoutRight)
"""
from __future__ import annotations

import numpy as np

CELL_BLOCK = 32
INTERP_MEMBERS = 18
FIELD_MEMBERS = 9
ACC_VALUES = 12
PARTICLE_REAL_MEMBERS = ("x", "y", "z", "ux", "uy", "uz", "w")

# field members (src/types.h:138-149)
F_EX, F_EY, F_EZ, F_CBX, F_CBY, F_CBZ, F_JFX, F_JFY, F_JFZ = range(9)


def real_dtype(precision) -> np.dtype:
    if precision in (4, np.float32) or np.dtype(precision) == np.float32:
        return np.dtype(np.float32)
    return np.dtype(np.float64)


def particle_block_bytes(real: np.dtype, vl: int) -> int:
    return vl * (7 * np.dtype(real).itemsize + 4)


def particle_list_bytes(n: int, real: np.dtype, vl: int) -> int:
    return -(-n // vl) * particle_block_bytes(real, vl)


def cell_array_bytes(num_cells: int, members: int, real: np.dtype) -> int:
    return -(-num_cells // CELL_BLOCK) * CELL_BLOCK * members * np.dtype(real).itemsize


def _particle_views(buf: np.ndarray, n: int, real: np.dtype, vl: int):
    real = np.dtype(real)
    nb = -(-n // vl)
    rs = real.itemsize
    blocks = buf[: nb * particle_block_bytes(real, vl)].reshape(nb, -1)
    mem = [blocks[:, m * vl * rs:(m + 1) * vl * rs].view(real) for m in range(7)]
    cell = blocks[:, 7 * vl * rs: 7 * vl * rs + 4 * vl].view(np.int32)
    return mem, cell


def pack_particles(p: dict, real=np.float32, vl: int = 32) -> np.ndarray:
    """dict of per-particle arrays (x, y, z, ux, uy, uz, w, cell) -> AoSoA bytes."""
    real = np.dtype(real)
    n = len(p["cell"])
    nb = -(-n // vl)
    buf = np.zeros(nb * particle_block_bytes(real, vl), np.uint8)
    mem, cell = _particle_views(buf, n, real, vl)
    pad = nb * vl - n
    for m, name in enumerate(PARTICLE_REAL_MEMBERS):
        a = np.asarray(p[name], dtype=real)
        mem[m][...] = np.concatenate([a, np.zeros(pad, real)]).reshape(nb, vl)
    c = np.asarray(p["cell"], dtype=np.int32)
    cell[...] = np.concatenate([c, np.zeros(pad, np.int32)]).reshape(nb, vl)
    return buf


def unpack_particles(buf: np.ndarray, n: int, real=np.float32, vl: int = 32) -> dict:
    real = np.dtype(real)
    buf = np.ascontiguousarray(buf).view(np.uint8).reshape(-1)
    mem, cell = _particle_views(buf, n, real, vl)
    out = {name: mem[m].reshape(-1)[:n].copy() for m, name in enumerate(PARTICLE_REAL_MEMBERS)}
    out["cell"] = cell.reshape(-1)[:n].copy()
    return out


def pack_cells(vals: np.ndarray, real=np.float32) -> np.ndarray:
    """(num_cells, members) -> AoSoA array of real (flat)."""
    real = np.dtype(real)
    nc, m = vals.shape
    nb = -(-nc // CELL_BLOCK)
    pad = np.zeros((nb * CELL_BLOCK, m), real)
    pad[:nc] = vals
    return np.ascontiguousarray(pad.reshape(nb, CELL_BLOCK, m).transpose(0, 2, 1)).reshape(-1)


def unpack_cells(arr: np.ndarray, num_cells: int, members: int) -> np.ndarray:
    """AoSoA array (flat) -> (num_cells, members)."""
    nb = -(-num_cells // CELL_BLOCK)
    a = np.asarray(arr).reshape(-1)[: nb * members * CELL_BLOCK].reshape(nb, members, CELL_BLOCK)
    return np.ascontiguousarray(a.transpose(0, 2, 1).reshape(nb * CELL_BLOCK, members)[:num_cells])


def voxel(x, y, z, nx, ny, ng=1):
    """VOXEL macro (src/types.h:195)."""
    return x + (nx + 2 * ng) * (y + (ny + 2 * ng) * z)


def rank_to_index(c, nx, ny, ng=1):
    """RANK_TO_INDEX (src/types.h:184-193) on the ghosted extents."""
    sx, sy = nx + 2 * ng, ny + 2 * ng
    iy, ix = np.divmod(c, sx)
    iz, iy = np.divmod(iy, sy)
    return ix, iy, iz
