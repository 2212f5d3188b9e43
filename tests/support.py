"""Seeded random states for the parity tests (test infrastructure)."""
from __future__ import annotations

import numpy as np

import oracle
from cabanapic_gb300 import layout as L


def random_state(nx=6, ny=5, nz=4, n=4000, seed=0, real=np.float32, crossing=0.3, vl=32,
                 sort=False, cdt=(0.45, 0.40, 0.35), qdt_2mc=-0.05, edge_cases=True, disorder=0.0):
    """Random interpolator + particles on an nx*ny*nz periodic grid.

    A fraction `crossing` of the particles gets large momenta (several face
    crossings per push); the rest move within their cell.  With edge_cases,
    some particles sit exactly on faces or have zero momentum components.
    With sort, particles are in cell order; `disorder` then moves that fraction
    of them to a random neighbouring interior cell without reordering (the
    state some steps after a sort)."""
    R = np.dtype(real).type
    rng = np.random.default_rng(seed)
    sx, sy, sz = nx + 2, ny + 2, nz + 2
    num_cells = sx * sy * sz
    # interpolator coefficients for every cell (ghost cells are never gathered)
    scale = np.array([0.2, 0.05, 0.05, 0.01] * 3 + [0.8, 0.1] * 3)
    interp_vals = (rng.standard_normal((num_cells, 18)) * scale).astype(R)
    interp = L.pack_cells(interp_vals, R)
    ix = rng.integers(1, nx + 1, n)
    iy = rng.integers(1, ny + 1, n)
    iz = rng.integers(1, nz + 1, n)
    cell = L.voxel(ix, iy, iz, nx, ny).astype(np.int32)
    off = rng.uniform(-1, 1, (3, n))
    big = rng.random(n) < crossing
    u = rng.standard_normal((3, n)) * np.where(big, 3.0, 0.004)
    if edge_cases and n >= 64:
        k = n // 16
        off[0, :k] = 1.0            # on the +x face, moving in or out
        off[1, k:2 * k] = -1.0      # on the -y face
        u[2, 2 * k:3 * k] = 0.0     # zero z motion (the 3.4e38 sentinel)
        u[:, 3 * k:3 * k + 8] = 0.0  # at rest
    w = rng.uniform(0.5, 1.5, n)
    p = dict(x=off[0], y=off[1], z=off[2], ux=u[0], uy=u[1], uz=u[2], w=w, cell=cell)
    if sort:
        order = np.argsort(cell, kind="stable")
        p = {k: v[order] for k, v in p.items()}
    if disorder > 0:
        moved = rng.random(n) < disorder
        jx, jy, jz = L.rank_to_index(p["cell"], nx, ny)
        d = rng.integers(-1, 2, (3, n))
        jx = np.where(moved, (jx - 1 + d[0]) % nx + 1, jx)
        jy = np.where(moved, (jy - 1 + d[1]) % ny + 1, jy)
        jz = np.where(moved, (jz - 1 + d[2]) % nz + 1, jz)
        p["cell"] = L.voxel(jx, jy, jz, nx, ny).astype(np.int32)
    p = {k: (v.astype(R) if k != "cell" else v) for k, v in p.items()}
    packed = L.pack_particles(p, R, vl)
    push_args = (R(qdt_2mc), R(cdt[0]), R(cdt[1]), R(cdt[2]), R(-1.0))
    return dict(particles=packed, host=p, interp=interp, interp_vals=interp_vals,
                push_args=push_args, ogrid=oracle.Oracle.grid(nx, ny, nz, 1), nx=nx, ny=ny, nz=nz,
                n=n, num_cells=num_cells, real=np.dtype(real), vl=vl)


def random_fields(nx, ny, nz, seed=0, real=np.float32, scale=1.0):
    """Random values for all 9 field members of every cell (AoSoA, flat)."""
    rng = np.random.default_rng(seed)
    nc = (nx + 2) * (ny + 2) * (nz + 2)
    vals = (rng.standard_normal((nc, 9)) * scale).astype(real)
    return L.pack_cells(vals, real), nc


def reorder_bound(acc_abs, count, eps):
    """Bound on |sum_a - sum_b| for two summation orders of the same terms:
    2 (k-1) eps sum|x| per accumulator (recursive summation error bound)."""
    k = np.maximum(count.astype(np.float64) - 1, 0)
    return 2.0 * k * eps * acc_abs.astype(np.float64) + 1e-30


def oracle_run(orc, deck, packed, steps, fields_init=None, out_state=None):
    """The reference's step sequence (example/example.cpp:221-266) in the
    oracle from a given packed particle list (and (num_cells, 9) initial field
    members, default zero); returns [steps, 2] energies accumulated in double.
    out_state, a dict, receives the final particle bytes and field members."""
    p = deck.derived()
    R = deck.R
    buf = packed.copy()
    nc = deck.num_cells
    g = orc.grid(deck.nx, deck.ny, deck.nz)
    if fields_init is None:
        fields = np.zeros(L.cell_array_bytes(nc, 9, R) // np.dtype(R).itemsize, R)
    else:
        fields = L.pack_cells(np.asarray(fields_init, R), R)
    interp = np.zeros(L.cell_array_bytes(nc, 18, R) // np.dtype(R).itemsize, R)
    h = R(0.5)
    out = []
    for _ in range(steps):
        orc.load_interpolator(fields, interp, g)
        acc = np.zeros((nc, 3, 4), R)
        orc.push(buf, deck.num_particles, deck.vl, interp, p["qdt_2mc"], p["cdt_dx"], p["cdt_dy"],
                 p["cdt_dz"], p["qsp"], acc, g)
        orc.unload_accumulator(fields, acc, g, p["dx"], p["dy"], p["dz"], p["dt"])
        orc.advance_b(fields, R(h * p["px"]), R(h * p["py"]), R(h * p["pz"]), g)
        orc.advance_e(fields, p["px"], p["py"], p["pz"], g, p["dt_eps0"])
        orc.advance_b(fields, R(h * p["px"]), R(h * p["py"]), R(h * p["pz"]), g)
        out.append(orc.energies(fields, g)[2:4])
    if out_state is not None:
        out_state["particles"] = buf
        out_state["fields"] = L.unpack_cells(fields, nc, 9)
    return np.array(out)


def history_deviation(a, b):
    """max_k |a_k - b_k| / max_k |b_k|, per column (E, B)."""
    return np.abs(a - b).max(axis=0) / np.abs(b).max(axis=0)


def global_position(p, nx, ny, nz):
    """Particle positions in half-cell units from the interior origin:
    X = 2 (ix - 1) + (x + 1), and likewise for y and z."""
    ix, iy, iz = L.rank_to_index(p["cell"].astype(np.int64), nx, ny)
    return (2.0 * (ix - 1) + (p["x"].astype(np.float64) + 1),
            2.0 * (iy - 1) + (p["y"].astype(np.float64) + 1),
            2.0 * (iz - 1) + (p["z"].astype(np.float64) + 1))


def assert_particles_close(got_bytes, ref_bytes, n, real, vl, nx, ny, nz, rtol=1e-5,
                           max_cell_flips=1e-3):
    """Per-particle tolerance check for the fused/approximate push: momenta to
    rtol relative to |u|, positions to rtol of a cell width (periodic, in
    global coordinates, so a particle that ends exactly on a face in one
    result and just across it in the other still compares equal), weights
    exact, and cell indices equal except for such face cases."""
    g = L.unpack_particles(got_bytes, n, real, vl)
    r = L.unpack_particles(ref_bytes, n, real, vl)
    assert np.array_equal(g["w"], r["w"])
    un = np.sqrt(sum(r[k].astype(np.float64) ** 2 for k in ("ux", "uy", "uz")))
    for k in ("ux", "uy", "uz"):
        d = np.abs(g[k].astype(np.float64) - r[k])
        assert np.all(d <= rtol * un + 1e-30), (k, (d / np.maximum(un, 1e-30)).max())
    for a, b, m in zip(global_position(g, nx, ny, nz), global_position(r, nx, ny, nz), (nx, ny, nz)):
        d = a - b
        d = (d + m) % (2 * m) - m  # periodic
        assert np.all(np.abs(d) <= 2 * rtol), np.abs(d).max()
    flips = np.count_nonzero(g["cell"] != r["cell"])
    assert flips <= max(1, max_cell_flips * n), flips
    return flips


def oracle_loss(orc, deck, packed, steps, fields_init=None, literal=True):
    """Field energy E + B (double) after `steps` steps of the reference's step
    sequence in the oracle, with its threaded push (deterministic for a fixed
    thread count).  literal=False (FP64): sqrt() for gamma, the function the
    FP64 adjoint differentiates."""
    p = deck.derived()
    R = deck.R
    buf = packed.copy()
    nc = deck.num_cells
    g = orc.grid(deck.nx, deck.ny, deck.nz)
    if fields_init is None:
        fields = np.zeros(L.cell_array_bytes(nc, 9, R) // np.dtype(R).itemsize, R)
    else:
        fields = L.pack_cells(np.asarray(fields_init, R), R)
    interp = np.zeros(L.cell_array_bytes(nc, 18, R) // np.dtype(R).itemsize, R)
    acc = np.zeros((nc, 3, 4), R)
    h = R(0.5)
    for _ in range(steps):
        orc.load_interpolator(fields, interp, g)
        acc.fill(0)
        orc.push_omp(buf, deck.num_particles, deck.vl, interp, p["qdt_2mc"], p["cdt_dx"], p["cdt_dy"],
                     p["cdt_dz"], p["qsp"], acc, g, literal=literal)
        orc.unload_accumulator(fields, acc, g, p["dx"], p["dy"], p["dz"], p["dt"])
        orc.advance_b(fields, R(h * p["px"]), R(h * p["py"]), R(h * p["pz"]), g)
        orc.advance_e(fields, p["px"], p["py"], p["pz"], g, p["dt_eps0"])
        orc.advance_b(fields, R(h * p["px"]), R(h * p["py"]), R(h * p["pz"]), g)
    e = orc.energies(fields, g)
    return float(e[2] + e[3])


def robust_central_difference(f, x0, steps, agree=1e-5):
    """Central differences of a piecewise-smooth f at x0 over the step sizes
    `steps`: the loss of a PIC run jumps where a particle's face crossing
    moves to another time step, and a difference whose +-h interval holds a
    jump measures the jump.  Returns the mean of the first two consecutive
    step sizes whose differences agree to `agree` relative, or raises."""
    fd = [(f(x0 + h) - f(x0 - h)) / (2 * h) for h in steps]
    for a, b in zip(fd, fd[1:]):
        if abs(a - b) <= agree * max(abs(a), abs(b)):
            return 0.5 * (a + b), fd
    raise AssertionError(f"no two central differences agree: {list(zip(steps, fd))}")
