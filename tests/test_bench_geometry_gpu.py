"""Parity at the benchmarked geometry: the time loop driven exactly as the
benchmark drives it (Simulation with the tiled push, captured step graphs and
a cell sort every 20 steps), checked against the oracle at the benchmark's
own sizes.

The tiled push's cell windows depend on the grid's row and plane strides
(130 and 16,900 voxels at 128^3) and on how far particles have drifted since
the last sort, so the checks run at those strides, right after a sort (step 1)
and after 19 steps of drift (step 19), against the reference's push
(src/push.h:65-299, src/move_p.h:93-371) restated in the oracle:

* the step's own push (default variant, graph-replayed): every particle
  within 1e-5 relative, accumulators within the summation-reordering bound;
* the exact variant on the same input (in place, tiled): particle AoSoA
  bytes identical to the oracle's;
* the energy history over 25 steps, across the sort at step 20, against the
  oracle's run from the same initial particles (1e-4 of the history's
  largest value).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from support import assert_particles_close, reorder_bound  # noqa: E402

pytestmark = pytest.mark.gpu

SORT_INTERVAL = 20


def _oracle_history_omp(orc, deck, packed, steps, fields_init=None):
    """The reference's step sequence (example/example.cpp:221-266) in the
    oracle with its OpenMP push (the same per-particle arithmetic as the
    serial push; accumulator sums in another order): [steps, 2] energies."""
    from cabanapic_gb300 import layout as L
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
    out = []
    for _ in range(steps):
        orc.load_interpolator(fields, interp, g)
        acc.fill(0)
        orc.push_omp(buf, deck.num_particles, deck.vl, interp, p["qdt_2mc"], p["cdt_dx"], p["cdt_dy"],
                     p["cdt_dz"], p["qsp"], acc, g)
        orc.unload_accumulator(fields, acc, g, p["dx"], p["dy"], p["dz"], p["dt"])
        orc.advance_b(fields, R(h * p["px"]), R(h * p["py"]), R(h * p["pz"]), g)
        orc.advance_e(fields, p["px"], p["py"], p["pz"], g, p["dt_eps0"])
        orc.advance_b(fields, R(h * p["px"]), R(h * p["py"]), R(h * p["pz"]), g)
        out.append(orc.energies(fields, g)[2:4])
    return np.array(out)


def _checked_step(sim, orc):
    """Runs sim.step() (a graph replay when the step does not sort, as in the
    benchmark) and checks its push against the oracle's push of the same
    input: the particles before the step and the interpolator the step loads
    from the fields before it.  Also pushes that input with the exact variant
    and checks it bit for bit.  Returns the number of cell-crossing
    particles."""
    from cabanapic_gb300 import pic
    from cabanapic_gb300.arrays import AccumulatorArray, InterpolatorArray, ParticleList
    d, p = sim.deck, sim.p
    R = d.R
    nc = d.num_cells
    assert sim.step_no % SORT_INTERVAL != 0, "the checked step must not sort"
    args = (p["qdt_2mc"], p["cdt_dx"], p["cdt_dy"], p["cdt_dz"], p["qsp"])
    # the step's inputs: the particles now and the interpolator of the fields now
    interp = InterpolatorArray(nc, R)
    pic.load_interpolator_array(sim.fields, interp, d.nx, d.ny, d.nz, d.num_ghosts)
    spare = ParticleList(d.num_particles, R, d.vl)
    spare.buf.copy_(sim.particles.buf)
    before = spare.buf.cpu().numpy()
    interp_host = interp.buf.cpu().numpy()

    sim.step()  # the benchmark's step: clear, push (default variant, tiled), field phase
    sim.check_status()
    after = sim.particles.download_bytes()
    acc_gpu = sim.accumulators.get()  # the field phase reads the deposits but does not clear them

    acc_exact = AccumulatorArray(nc, R)
    pic.push(spare, interp, *args, acc_exact, None, d.nx, d.ny, d.nz, d.num_ghosts, d.boundary, exact=True,
             tiles=True)
    pic.check_status()
    after_exact = spare.download_bytes()
    acc_exact_host = acc_exact.get()
    del spare, interp, acc_exact

    ref = before.copy()
    acc = np.zeros((nc, 3, 4), R)
    acc_abs = np.zeros((nc, 3, 4), R)
    cnt = np.zeros((nc, 3, 4), np.int32)
    crossers = orc.push(ref, d.num_particles, d.vl, interp_host, *args, acc, orc.grid(d.nx, d.ny, d.nz),
                        acc_abs=acc_abs, acc_count=cnt)
    eps = np.finfo(R).eps
    bound = reorder_bound(acc_abs, cnt, eps)

    assert np.array_equal(after_exact, ref), "exact variant: particle AoSoA bytes differ from the oracle"
    err = np.abs(acc_exact_host.astype(np.float64) - acc)
    assert np.all(err <= bound), f"exact variant: accumulator error {err.max():.3e} above the bound"

    assert_particles_close(after, ref, d.num_particles, R, d.vl, d.nx, d.ny, d.nz)
    bound = bound + 1e-5 * acc_abs + 1e-6 * float(acc_abs.max())
    err = np.abs(acc_gpu.astype(np.float64) - acc)
    assert np.all(err <= bound), f"default variant: accumulator error {err.max():.3e} above the bound"
    return crossers


def _run_geometry(orc, deck, host_packed=None, fields=None):
    from cabanapic_gb300.simulation import Simulation
    sim = Simulation(deck, host_packed, sort_interval=SORT_INTERVAL, max_steps=30, graphs=True,
                     fields=fields)
    assert sim.tiles and not sim.exact  # the benchmark's push
    init = sim.particles.download_bytes() if host_packed is None else host_packed
    sim.step()  # step 0: sort, then push (eager)
    sim.prepare_graphs()
    n = deck.num_particles
    c1 = _checked_step(sim, orc)  # step 1, right after the sort
    sim.run(SORT_INTERVAL - 2 - 1)  # steps 2..18, graph replays
    c19 = _checked_step(sim, orc)  # step 19: 19 steps of drift
    sim.run(5)  # steps 20..24: sort at step 20
    assert sim.step_no == 25
    sim.check_status()
    e_gpu = sim.energies()
    del sim
    torch.cuda.empty_cache()
    e_ref = _oracle_history_omp(orc, deck, init, 25, fields_init=fields)
    return c1 / n, c19 / n, e_gpu, e_ref


def test_thermal_128_cubed_64ppc_matches_oracle(orc):
    """The benchmark's workload: 128^3 cells x 64 ppc (134,217,728 particles),
    FP32, the seeded device loader, sort every 20 steps."""
    from cabanapic_gb300 import decks
    deck = decks.thermal(n=128, ppc=64, precision=4, num_steps=25)
    f1, f19, e_gpu, e_ref = _run_geometry(orc, deck)
    assert f1 > 0.01 and f19 > 0.01  # the mover path was exercised
    dev = np.abs(e_gpu - e_ref).max(axis=0) / np.abs(e_ref).max(axis=0)
    assert np.all(dev < 1e-4), dev


def test_diocotron_96x96x64_matches_oracle(orc):
    """The diocotron column at its benchmarked size: 96 x 96 x 64 cells, 128
    particles per cell of the annulus, E x B loading in the t = 0 field."""
    from cabanapic_gb300 import decks
    deck = decks.diocotron(precision=4, num_steps=25)
    host, fields = decks.diocotron_state(deck, packed=True)
    f1, f19, e_gpu, e_ref = _run_geometry(orc, deck, host, fields)
    assert f1 > 0.01 and f19 > 0.01
    dev = np.abs(e_gpu - e_ref).max(axis=0) / np.abs(e_ref).max(axis=0)
    assert np.all(dev < 1e-4), dev
