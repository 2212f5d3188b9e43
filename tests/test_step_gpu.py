"""Whole-step parity: the GPU time loop (Simulation and the C++ minipic
driver) against the oracle and against the reference's golden energy
histories, with the reference's own acceptance rule."""
import os
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from conftest import gold_path  # noqa: E402
from oracle import energy_rule  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu_runs():
    from cabanapic_gb300 import decks
    from cabanapic_gb300.simulation import Simulation
    out = {}
    for prec in (4, 8):
        deck = decks.two_stream_em(precision=prec, num_steps=6000)
        sim = Simulation(deck)
        sim.run(6000)
        sim.check_status()
        out[prec] = (sim.energies(), deck.derived())
    return out


def test_double_gpu_reproduces_double_gold(gpu_runs):
    e, _ = gpu_runs[8]
    gold = np.loadtxt(gold_path("double"))
    rel = np.abs(e / gold[:, 2:4] - 1)
    # the gold prints 7 significant digits
    assert rel.max() < 2e-6, rel.max()


@pytest.mark.parametrize("prec,kind", [(4, "float"), (8, "double")])
def test_gpu_passes_reference_acceptance_rule(gpu_runs, prec, kind):
    e, p = gpu_runs[prec]
    ours = energy_rule.format_history(e, float(p["dt"]))
    gold = open(gold_path(kind)).read().splitlines()
    (e_ok, e_err, _, _), (b_ok, b_err, _, _) = energy_rule.two_stream_em_check(gold, ours)
    assert e_ok, e_err
    assert b_ok, b_err


def test_float_gpu_tracks_oracle_early(gpu_runs, orc):
    e, _ = gpu_runs[4]
    ref, _ = orc.run_two_stream_em(200, 4)
    rel = np.abs(e[:200] / ref[:, 2:4] - 1)
    assert rel[:50].max() < 1e-5, rel[:50].max()
    assert rel.max() < 1e-3, rel.max()


def test_thermal_3d_steps_track_oracle(orc):
    """8^3 cells x 8 ppc thermal plasma, 20 full steps on the GPU and in the
    oracle from the same initial state: field energies agree closely."""
    from cabanapic_gb300 import decks, layout as L
    from cabanapic_gb300.simulation import Simulation
    deck = decks.thermal(n=8, ppc=8, uth=0.2, dx=0.1, num_steps=20, seed=3)
    p = deck.derived()
    host = decks.thermal_particles(deck)
    sim = Simulation(deck, host)
    sim.run(20)
    sim.check_status()
    e_gpu = sim.energies()
    # oracle, same sequence
    R = deck.R
    buf = L.pack_particles(host, R, 32)
    nc = deck.num_cells
    g = orc.grid(deck.nx, deck.ny, deck.nz)
    fields = np.zeros(L.cell_array_bytes(nc, 9, R) // R().itemsize, R)
    interp = np.zeros(L.cell_array_bytes(nc, 18, R) // R().itemsize, R)
    e_ref = []
    for _ in range(20):
        orc.load_interpolator(fields, interp, g)
        acc = np.zeros((nc, 3, 4), R)
        orc.push(buf, deck.num_particles, 32, interp, p["qdt_2mc"], p["cdt_dx"], p["cdt_dy"],
                 p["cdt_dz"], p["qsp"], acc, g)
        orc.unload_accumulator(fields, acc, g, p["dx"], p["dy"], p["dz"], p["dt"])
        h = R(0.5)
        orc.advance_b(fields, R(h * p["px"]), R(h * p["py"]), R(h * p["pz"]), g)
        orc.advance_e(fields, p["px"], p["py"], p["pz"], g, p["dt_eps0"])
        orc.advance_b(fields, R(h * p["px"]), R(h * p["py"]), R(h * p["pz"]), g)
        e_ref.append(orc.energies(fields, g)[2:4])
    e_ref = np.array(e_ref)
    rel = np.abs(e_gpu / e_ref - 1)
    assert rel.max() < 1e-4, rel.max()


@pytest.mark.parametrize("exe,kind", [("minipic", "float"), ("minipic_f64", "double")])
def test_cpp_driver_passes_reference_rule(tmp_path, exe, kind):
    """The C++ time loop written against include/cpic/cabana.hpp (the
    reference's push() signature and containers) runs the 2stream-em deck and
    its energies.txt passes the reference's regression rule."""
    from cabanapic_gb300 import build
    path = os.path.join(build.OUT, exe)
    assert os.path.exists(path), "C++ driver not built"
    out = tmp_path / "energies.txt"
    r = subprocess.run([path, "6000", str(out)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    ours = out.read_text().splitlines()
    assert len(ours) == 6000
    gold = open(gold_path(kind)).read().splitlines()
    (e_ok, e_err, _, _), (b_ok, b_err, _, _) = energy_rule.two_stream_em_check(gold, ours)
    assert e_ok, e_err
    assert b_ok, b_err
