"""Pins the CPU oracle against the reference's own golden energy histories.

The reference's regression test (tests/energy_comparison/2stream-em.cxx) runs
the 2stream-em deck for 6000 steps and compares E and B energies against
energies_gold.2stream-em.{float,double} with 10% relative tolerance on rows
3581..4880.  The oracle must pass that rule, and in double precision it must
reproduce every printed digit of the double gold.
"""
import numpy as np
import pytest

from oracle import energy_rule
from conftest import gold_path


@pytest.fixture(scope="module")
def runs(orc):
    return {prec: orc.run_two_stream_em(6000, prec) for prec in (4, 8)}


def test_double_oracle_reproduces_double_gold_to_print_precision(runs):
    out, par = runs[8]
    gold = np.loadtxt(gold_path("double"))
    assert gold.shape == (6000, 4)
    # the gold prints 7 significant digits: relative rounding <= 5e-7
    rel_e = np.abs(out[:, 0] / gold[:, 2] - 1)
    rel_b = np.abs(out[:, 1] / gold[:, 3] - 1)
    assert rel_e.max() < 1e-6, rel_e.max()
    assert rel_b.max() < 1e-6, rel_b.max()
    # the time column: row k is printed with time k*dt (%f)
    assert np.allclose(gold[:, 1], np.arange(6000) * par["dt"], atol=1e-6)


def test_float_oracle_tracks_float_gold_in_linear_phase(runs):
    out, _ = runs[4]
    gold = np.loadtxt(gold_path("float"))
    rel_e = np.abs(out[:300, 0] / gold[:300, 2] - 1)
    rel_b = np.abs(out[:300, 1] / gold[:300, 3] - 1)
    # row 0 agrees to the gold's print precision; float summation order of the
    # energy reduction is the only known source of the small drift after it
    assert rel_e[0] < 5e-6 and rel_b[0] < 5e-6
    assert rel_e.max() < 2e-3 and rel_b.max() < 2e-3


@pytest.mark.parametrize("prec,kind", [(4, "float"), (8, "double")])
def test_reference_acceptance_rule(runs, prec, kind):
    out, par = runs[prec]
    ours = energy_rule.format_history(out[:, :2], par["dt"])
    gold = open(gold_path(kind)).read().splitlines()
    (e_ok, e_err, _, _), (b_ok, b_err, _, _) = energy_rule.two_stream_em_check(gold, ours)
    assert e_ok, e_err
    assert b_ok, b_err


def test_energy_rule_detects_a_planted_error(runs):
    out, par = runs[8]
    bad = out[:, :2].copy()
    bad[4000, 0] *= 1.2   # 20% error in one E row of the checked window
    ours = energy_rule.format_history(bad, par["dt"])
    gold = open(gold_path("double")).read().splitlines()
    (e_ok, e_err, line, _), (b_ok, _, _, _) = energy_rule.two_stream_em_check(gold, ours)
    assert not e_ok and line == 4000 and b_ok


def test_compare_error_absolute_branch():
    ok, err = energy_rule.compare_error(0.0, 1e-17, 0.1)
    assert ok and err == 1e-17
    ok, _ = energy_rule.compare_error(0.0, 1e-15, 0.1)
    assert not ok


@pytest.mark.parametrize("fold", [False, True])
def test_oracle_es_solver_restates_the_reference(orc, fold):
    """src/fields.h:400-436 / 511-544: E -= cj J over every cell (ghosts
    included); the 1-D variant folds the jf ghosts first."""
    from support import random_fields
    nx, ny, nz = 9, 1, 1
    f, nc = random_fields(nx, ny, nz, seed=4, real=np.float64)
    g = orc.grid(nx, ny, nz)
    got = f.copy()
    orc.es_advance_e(got, g, 0.25, fold)
    src = f.copy()
    if fold:
        orc.current_fold(src, g)
    from cabanapic_gb300 import layout as L
    v = L.unpack_cells(src, nc, 9)
    v[:, 0:3] -= 0.25 * v[:, 6:9]
    assert np.allclose(L.unpack_cells(got, nc, 9), v, rtol=0, atol=1e-15)
    e = L.unpack_cells(got, nc, 9)[:, 0:3]
    assert abs(orc.es_energy(got, g) - 0.5 * (e ** 2).sum()) < 1e-12 * (e ** 2).sum()
