"""The diocotron column (uniform axial B, E x B-drifting annulus loaded from
the t = 0 Poisson field): the GPU step sequence against the oracle from the
same initial particles and fields, and charge conservation under its heavy
cell crossing."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from support import oracle_run  # noqa: E402

pytestmark = pytest.mark.gpu


def _deck(precision):
    from cabanapic_gb300 import decks
    return decks.diocotron(n=(24, 24, 8), ppc=32, dx=0.2, precision=precision, num_steps=40)


def test_fp64_gpu_matches_oracle_from_initial_fields(orc):
    from cabanapic_gb300 import decks, layout as L
    from cabanapic_gb300.simulation import Simulation
    deck = _deck(8)
    host, fields = decks.diocotron_state(deck)
    sim = Simulation(deck, host, fields=fields, exact=True, sort_interval=10)
    sim.run(40)
    sim.check_status()
    state = {}
    ref = oracle_run(orc, deck, L.pack_particles(host, np.float64, 32), 40, fields_init=fields,
                     out_state=state)
    rel = np.abs(sim.energies() / ref - 1)
    assert rel.max() < 1e-10, rel.max()
    # the GPU sorted its particles every 10 steps: compare as sets of states
    g = sim.download_particles()
    o = L.unpack_particles(state["particles"], deck.num_particles, np.float64, 32)
    key = lambda p: np.lexsort((p["uz"], p["uy"], p["ux"], p["cell"]))  # noqa: E731
    gi, oi = key(g), key(o)
    assert np.array_equal(g["cell"][gi], o["cell"][oi])
    for k in ("x", "y", "z", "ux", "uy", "uz"):
        np.testing.assert_allclose(g[k][gi], o[k][oi], rtol=0, atol=1e-11)


@pytest.mark.parametrize("precision", [4, 8])
def test_charge_conserved_with_heavy_crossing(precision):
    from cabanapic_gb300 import decks, pic
    from cabanapic_gb300.simulation import Simulation
    deck = _deck(precision)
    p = deck.derived()
    sim = Simulation(deck, sort_interval=20)
    D = pic.Diagnostics(deck.num_cells)
    args = (deck.nx, deck.ny, deck.nz, 1)
    dxyz = (float(p["dx"]), float(p["dy"]), float(p["dz"]))
    rho0 = D.charge_density(sim.particles, *args, float(p["qsp"]), *dxyz).clone()
    r0 = torch.zeros(deck.num_cells, dtype=torch.float64, device="cuda")
    D.gauss_residual(sim.fields, rho0, *args, *dxyz, eps0=float(p["eps"]), resid=r0)
    rho_max = float(rho0.abs().max())
    # t = 0: div E - rho is the uniform background alone
    bg = r0.view(deck.nz + 2, deck.ny + 2, deck.nx + 2)[1:-1, 1:-1, 1:-1]
    assert float((bg - bg.mean()).abs().max()) < (1e-10 if precision == 8 else 1e-5) * rho_max
    crossers = 0
    worst = 0.0
    for _ in range(40):
        before = sim.particles.download()["cell"] if crossers == 0 else None
        sim.step()
        if before is not None:
            crossers = int((sim.particles.download()["cell"] != before).sum())
        rho = D.charge_density(sim.particles, *args, float(p["qsp"]), *dxyz)
        out = D.gauss_residual(sim.fields, rho, *args, *dxyz, eps0=float(p["eps"]), ref=r0).cpu().numpy()
        worst = max(worst, out[0] / rho_max)
    sim.check_status()
    assert crossers > 0.01 * deck.num_particles  # particles change cell every step
    assert worst < (1e-11 if precision == 8 else 2e-5), worst
