"""Host-side layout packing and deck arithmetic, checked against the oracle."""
import numpy as np
import pytest

from cabanapic_gb300 import decks, layout as L


@pytest.mark.parametrize("real,vl", [(np.float32, 32), (np.float32, 16), (np.float64, 32), (np.float64, 16)])
def test_particle_pack_roundtrip(real, vl):
    rng = np.random.default_rng(1)
    n = 1000 + vl // 2
    p = {k: rng.standard_normal(n).astype(real) for k in L.PARTICLE_REAL_MEMBERS}
    p["cell"] = rng.integers(0, 1 << 20, n).astype(np.int32)
    buf = L.pack_particles(p, real, vl)
    assert buf.nbytes == L.particle_list_bytes(n, real, vl)
    q = L.unpack_particles(buf, n, real, vl)
    for k in p:
        assert np.array_equal(p[k], q[k])
    # member m of particle i sits at (i//vl)*block + m*vl*rs + (i%vl)*rs
    rs = np.dtype(real).itemsize
    i = 777
    off = (i // vl) * L.particle_block_bytes(real, vl) + 3 * vl * rs + (i % vl) * rs
    assert buf[off:off + rs].view(real)[0] == p["ux"][i]
    off = (i // vl) * L.particle_block_bytes(real, vl) + 7 * vl * rs + (i % vl) * 4
    assert buf[off:off + 4].view(np.int32)[0] == p["cell"][i]


def test_cell_pack_roundtrip():
    rng = np.random.default_rng(2)
    v = rng.standard_normal((1001, 18)).astype(np.float32)
    a = L.pack_cells(v, np.float32)
    assert a.size == L.cell_array_bytes(1001, 18, np.float32) // 4
    assert np.array_equal(L.unpack_cells(a, 1001, 18), v)
    c, m = 555, 13
    assert a[(c // 32) * 18 * 32 + m * 32 + c % 32] == v[c, m]


def test_voxel_and_rank_to_index():
    nx, ny, nz = 7, 5, 3
    x, y, z = np.meshgrid(np.arange(nx + 2), np.arange(ny + 2), np.arange(nz + 2), indexing="ij")
    c = L.voxel(x, y, z, nx, ny)
    assert c.max() == (nx + 2) * (ny + 2) * (nz + 2) - 1
    ix, iy, iz = L.rank_to_index(c, nx, ny)
    assert np.array_equal(ix, x) and np.array_equal(iy, y) and np.array_equal(iz, z)


@pytest.mark.parametrize("prec", [4, 8])
def test_two_stream_em_deck_matches_oracle(orc, prec):
    d = decks.two_stream_em(prec)
    p = d.derived()
    _, par = orc.run_two_stream_em(1, prec)
    for k in ("dt", "dx", "dy", "dz", "qdt_2mc", "we", "py"):
        assert float(p[k]) == par[k], k
    assert float(p["len_y"]) == par["len_y"]


@pytest.mark.parametrize("prec", [4, 8])
def test_default_initializer_matches_oracle_bitwise(orc, prec):
    d = decks.two_stream_em(prec)
    p = d.derived()
    R = d.R
    buf = L.pack_particles(decks.default_particles(d), R, 32)
    ref = np.zeros_like(buf)
    orc.default_particle_init(ref, d.num_particles, 32, d.nx, d.ny, p["dxp"], d.nppc, p["we"], R(d.v0), R)
    assert np.array_equal(buf, ref)


def test_thermal_initializer_shapes():
    d = decks.thermal(n=4, ppc=8, num_steps=1)
    p = decks.thermal_particles(d)
    assert len(p["cell"]) == 4 ** 3 * 8
    assert np.all(np.diff(p["cell"]) >= 0)  # cell order
    assert np.abs(p["x"]).max() <= 1 and np.abs(p["y"]).max() <= 1
    ix, iy, iz = L.rank_to_index(p["cell"], 4, 4)
    assert ix.min() == 1 and ix.max() == 4 and iz.max() == 4
    np.testing.assert_allclose(p["w"].sum(), 1.0 * d.len_x_global ** 3, rtol=1e-5)
    buf = decks.thermal_particles(d, packed=True)
    assert np.array_equal(L.unpack_particles(buf, len(p["cell"]))["ux"], p["ux"])


def test_courant_length():
    R = np.float32
    cl = decks.courant_length(1.0, 2.0, 3.0, 10, 20, 30, R)
    w = (10 / 1.0) ** 2 + (20 / 2.0) ** 2 + (30 / 3.0) ** 2
    assert abs(float(cl) - (1 / w) ** 0.5) < 1e-7


def test_product_energy_rule_matches_the_oracle_restatement(orc):
    """cabanapic_gb300.energies (user-facing) against oracle.energy_rule on the
    reference's gold files and the oracle's own history."""
    from cabanapic_gb300 import energies
    from conftest import gold_path
    from oracle import energy_rule
    out, par = orc.run_two_stream_em(6000, 8)
    ours = energies.history_lines(out[:, :2], par["dt"])
    assert ours == energy_rule.format_history(out[:, :2], par["dt"])
    for kind in ("float", "double"):
        gold = open(gold_path(kind)).read().splitlines()
        (pe, ee, le), (pb, eb, lb) = energies.two_stream_em_rule(gold, ours)
        (qe, fe, me, _), (qb, fb, mb, _) = energy_rule.two_stream_em_check(gold, ours)
        assert (pe, pb) == (qe, qb) and (ee, eb) == (fe, fb) and (le, lb) == (me, mb)


def test_diocotron_initial_state():
    """The column's t = 0 field solves the discrete Gauss law (backward-difference
    div E at the nodes) for the particles' node charge plus the uniform
    background; particles sit in the annulus, in cell order, drifting along
    E x B."""
    from oracle import diagnostics
    nx, ny, nz = 32, 32, 8
    d = decks.diocotron(n=(nx, ny, nz), ppc=16, dx=0.2, precision=8)
    p, f = decks.diocotron_state(d)
    par = d.derived()
    dx, dy, dz = (float(par[k]) for k in ("dx", "dy", "dz"))
    assert len(p["cell"]) == d.num_particles and d.num_particles % 32 == 0
    assert np.all(np.diff(p["cell"]) >= 0)
    rho = diagnostics.charge_density(p, nx, ny, nz, float(par["qsp"]), dx, dy, dz)[1:-1, 1:-1, 1:-1]
    res = diagnostics.div_e(f, nx, ny, nz, dx, dy, dz) - (rho - rho.mean())
    assert np.abs(res).max() < 1e-10 * np.abs(rho).max()
    # the total charge is -n0 x annulus volume
    rad = d.extra["radius"]
    vol = np.pi * (0.35 ** 2 - 0.20 ** 2) * rad * rad * d.len_z_global
    np.testing.assert_allclose(rho.sum() * dx * dy * dz, -vol, rtol=1e-3)
    # u is perpendicular to E at the particle (cold E x B drift), z momentum zero
    assert np.all(p["uz"] == 0)
    X, Y, _ = (a * dx / 2 for a in _global(p, nx, ny, nz))
    r = np.hypot(X - d.len_x_global / 2, Y - d.len_y_global / 2) / rad
    assert r.min() > 0.2 - 1e-9 and r.max() < 0.35 + 1e-9
    # the drift goes around the axis (the field of the periodic, discretised
    # column is radial up to its images and the l = 3 ripple)
    radial = (p["ux"] * (X - d.len_x_global / 2) + p["uy"] * (Y - d.len_y_global / 2)) / (r * rad)
    speed = np.hypot(p["ux"], p["uy"])
    assert np.abs(radial).mean() < 0.15 * speed.mean()


def _global(p, nx, ny, nz):
    ix, iy, iz = L.rank_to_index(p["cell"].astype(np.int64), nx, ny)
    return (2.0 * (ix - 1) + (p["x"].astype(np.float64) + 1),
            2.0 * (iy - 1) + (p["y"].astype(np.float64) + 1),
            2.0 * (iz - 1) + (p["z"].astype(np.float64) + 1))


def test_diocotron_slab_matches_reference_initializers():
    """decks/dioctron_3d.cxx: 64 x 64 x 1, 5 per cell, strip |y| < a, first z
    layer, at rest; E_y clamped shear and cB_z = sqrt(20)."""
    d = decks.diocotron_slab(precision=8)
    p, f = decks.diocotron_slab_state(d)
    assert d.num_particles == 64 * 64 * 5
    ix, iy, iz = L.rank_to_index(p["cell"].astype(np.int64), 64, 64)
    assert np.all(iz == 1) and np.all(p["z"] == 0) and np.all(p["ux"] == 0)
    ypos = -0.8 + (iy - 1 + (p["y"] + 1) / 2) * 0.025
    assert np.abs(ypos).max() <= 0.1 + 1e-12
    F = f.reshape(3, 66, 66, 9)
    assert np.all(F[..., 5] == np.sqrt(20.0))
    yc = -0.8 + (np.arange(66) - 0.5) * 0.025
    np.testing.assert_array_equal(F[1, :, 7, 1], np.where(yc < -0.1, 0.1, np.where(yc > 0.1, -0.1, -yc)))


def test_philox_known_answers():
    """Philox4x32-10 against the known-answer vectors published with the
    generator (Random123: zero counter and key; all-ones; the pi digits)."""
    kats = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
            ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
            ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
             (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for ctr, key, want in kats:
        got = decks.philox4x32_10(*(np.array([c], np.uint64) for c in ctr), *key)
        assert tuple(int(g[0]) for g in got) == want


@pytest.mark.parametrize("prec", [4, 8])
def test_thermal_stream_is_keyed_by_particle_index(prec):
    """The thermal loader's values depend only on (seed, particle index): a
    prefix sample equals the start of the full list, and the Maxwellian and
    uniform statistics hold."""
    d = decks.thermal(n=8, ppc=64, precision=prec, num_steps=1, seed=99)
    full = decks.thermal_particles(d)
    part = decks.thermal_particles(d, n_sample=1000)
    for k in full:
        assert np.array_equal(full[k][:1000], part[k])
    n = len(full["x"])
    for k in ("x", "y", "z"):
        assert full[k].min() >= -1 and full[k].max() < 1
        assert abs(full[k].astype(np.float64).mean()) < 4 / np.sqrt(3 * n)
    for k in ("ux", "uy", "uz"):
        u = full[k].astype(np.float64)
        assert abs(u.mean()) < 4 * 0.05 / np.sqrt(n)
        assert abs(u.std() / 0.05 - 1) < 4 / np.sqrt(2 * n)
    other = decks.thermal_particles(decks.thermal(n=8, ppc=64, precision=prec, num_steps=1, seed=100),
                                    n_sample=1000)
    assert not np.array_equal(other["ux"], part["ux"])
