"""FP64 diagnostics (charge density, Gauss residual, kinetic energy) against
their numpy restatement, and the property they exist to measure: the push's
charge-conserving deposit plus the Yee update keep div E - rho/eps0 constant
in time, to round-off."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from support import random_fields, random_state  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("real,vl,sort", [(np.float32, 32, True), (np.float32, 16, False),
                                          (np.float64, 32, False)])
def test_charge_density_matches_numpy(real, vl, sort):
    from cabanapic_gb300 import pic
    from oracle import diagnostics as od
    nx, ny, nz = 7, 5, 6
    st = random_state(nx=nx, ny=ny, nz=nz, n=30011, seed=3, real=real, vl=vl, sort=sort)
    P = pic.ParticleList(st["n"], real, vl).upload(st["particles"])
    D = pic.Diagnostics(st["num_cells"])
    dx, dy, dz = 0.3, 0.25, 0.2
    rho = D.charge_density(P, nx, ny, nz, 1, -1.0, dx, dy, dz).cpu().numpy()
    pic.check_status()
    ref = od.charge_density(st["host"], nx, ny, nz, -1.0, dx, dy, dz).reshape(-1)
    scale = np.abs(ref).max()
    assert np.allclose(rho, ref, rtol=1e-12, atol=1e-12 * scale)
    # total charge is conserved by the fold
    assert np.isclose(rho.sum() * dx * dy * dz, -st["host"]["w"].astype(np.float64).sum(), rtol=1e-12)


@pytest.mark.parametrize("real", [np.float32, np.float64])
def test_gauss_residual_matches_numpy(real):
    from cabanapic_gb300 import layout as L, pic
    from oracle import diagnostics as od
    nx, ny, nz = 9, 4, 6
    f, nc = random_fields(nx, ny, nz, seed=8, real=real)
    F = pic.FieldArray(nc, real)
    F.buf.copy_(torch.from_numpy(f))
    rng = np.random.default_rng(2)
    rho = rng.standard_normal(nc)
    refr = rng.standard_normal(nc)
    D = pic.Diagnostics(nc)
    resid = torch.zeros(nc, dtype=torch.float64, device="cuda")
    dx, dy, dz, eps0 = 0.3, 0.25, 0.2, 1.7
    out = D.gauss_residual(F, torch.from_numpy(rho).cuda(), nx, ny, nz, 1, dx, dy, dz, eps0,
                           ref=torch.from_numpy(refr).cuda(), resid=resid).cpu().numpy()
    cells = L.unpack_cells(f, nc, 9)
    r = od.gauss_residual(cells, rho.reshape(nz + 2, ny + 2, nx + 2), nx, ny, nz, dx, dy, dz, eps0)
    r = r - refr.reshape(nz + 2, ny + 2, nx + 2)[1:nz + 1, 1:ny + 1, 1:nx + 1]
    got = resid.cpu().numpy().reshape(nz + 2, ny + 2, nx + 2)[1:nz + 1, 1:ny + 1, 1:nx + 1]
    assert np.allclose(got, r, rtol=1e-12, atol=1e-12)
    assert np.isclose(out[0], np.abs(r).max(), rtol=1e-12)
    assert np.isclose(out[1], (r ** 2).sum(), rtol=1e-10)
    rq = rho.reshape(nz + 2, ny + 2, nx + 2)[1:nz + 1, 1:ny + 1, 1:nx + 1] / eps0
    assert np.isclose(out[2], (rq ** 2).sum(), rtol=1e-10)


@pytest.mark.parametrize("real,vl", [(np.float32, 32), (np.float64, 16)])
def test_kinetic_energy_matches_numpy(real, vl):
    from cabanapic_gb300 import pic
    from oracle import diagnostics as od
    st = random_state(n=12345, seed=5, real=real, vl=vl)
    P = pic.ParticleList(st["n"], real, vl).upload(st["particles"])
    D = pic.Diagnostics(st["num_cells"])
    ke = float(D.kinetic_energy(P, mc2=2.5).cpu()[0])
    assert np.isclose(ke, od.kinetic_energy(st["host"], 2.5), rtol=1e-12)


@pytest.mark.parametrize("precision,exact", [(8, True), (8, False), (4, True), (4, False)])
def test_charge_is_conserved_over_steps(precision, exact):
    """div E - rho/eps0 stays at its initial value to round-off over 12 steps
    of a thermal plasma with many cell crossings."""
    from cabanapic_gb300 import decks, pic
    from cabanapic_gb300.simulation import Simulation
    deck = decks.thermal(n=8, ppc=16, uth=0.25, dx=0.1, precision=precision, num_steps=12, seed=11)
    p = deck.derived()
    sim = Simulation(deck, exact=exact, sort_interval=5)
    D = pic.Diagnostics(deck.num_cells)
    args = (deck.nx, deck.ny, deck.nz, 1)
    dxyz = (float(p["dx"]), float(p["dy"]), float(p["dz"]))
    rho0 = D.charge_density(sim.particles, *args, float(p["qsp"]), *dxyz).clone()
    r0 = torch.zeros(deck.num_cells, dtype=torch.float64, device="cuda")
    D.gauss_residual(sim.fields, rho0, *args, *dxyz, eps0=float(p["eps"]), resid=r0)
    rho_max = float(rho0.abs().max())
    worst = 0.0
    for _ in range(12):
        sim.step()
        rho = D.charge_density(sim.particles, *args, float(p["qsp"]), *dxyz)
        out = D.gauss_residual(sim.fields, rho, *args, *dxyz, eps0=float(p["eps"]), ref=r0).cpu().numpy()
        worst = max(worst, out[0] / rho_max)
    sim.check_status()
    pic.check_status()
    # FP64: round-off; FP32: single-precision fields and offsets
    assert worst < (1e-12 if precision == 8 else 2e-5), worst
