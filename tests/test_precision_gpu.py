"""Precision study support: the full-FP64 GPU build reproduces the FP64 oracle
(the reference's real_t = double arithmetic) to round-off on the same initial
state, so it can stand for the oracle at the study's full size; and a small
FP32-vs-FP64 study runs end to end with sane error levels."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from support import oracle_run  # noqa: E402

pytestmark = pytest.mark.gpu


def test_fp64_gpu_matches_fp64_oracle(orc):
    from cabanapic_gb300 import decks, layout as L
    from cabanapic_gb300.simulation import Simulation
    deck = decks.thermal(n=8, ppc=16, uth=0.1, dx=0.1, precision=8, num_steps=30, seed=9)
    host = decks.thermal_particles(deck)
    sim = Simulation(deck, host, exact=True)
    sim.run(30)
    sim.check_status()
    ref = oracle_run(orc, deck, L.pack_particles(host, np.float64, 32), 30)
    rel = np.abs(sim.energies() / ref - 1)
    assert rel.max() < 1e-11, rel.max()


def test_small_precision_study_runs():
    from cabanapic_gb300 import precision
    out = precision.run(cells=16, ppc=8, steps=40, seed=3, sample_every=10)
    f = out["final"]
    assert out["pushes_per_s_fp32"] > 0 and out["pushes_per_s_fp64"] > 0
    assert 0 < out["max_field_l2_rel"] < 1e-2
    assert abs(f["energy_drift_fp64"]) < 1e-2
    assert f["charge_err_fp64"] < 1e-11
    assert f["charge_err_fp32"] < 1e-4
    assert 0 <= out["field_energy_rel_err_max"] < 1.0
    assert out["field_energy_level_rel_diff_second_half"] < 0.2
