"""Self-checks of the oracle itself, on the CPU: the serial step is
deterministic, its charge-conserving deposit and Yee update keep
div E - rho/eps0 at its initial value to round-off in FP64, and the OpenMP
push (per-thread accumulator copies, the timed CPU baseline) moves every
particle exactly as the serial push and sums the same currents up to the
order of the additions."""
import numpy as np
import pytest

from cabanapic_gb300 import decks, layout as L
from oracle import diagnostics as od
from support import oracle_run, reorder_bound


def _thermal(precision, n=6, ppc=8, steps=8):
    deck = decks.thermal(n=n, ppc=ppc, uth=0.25, dx=0.1, precision=precision, num_steps=steps, seed=17)
    return deck, L.pack_particles(decks.thermal_particles(deck), deck.R, deck.vl)


@pytest.mark.parametrize("precision", [4, 8])
def test_serial_oracle_step_is_deterministic(orc, precision):
    deck, packed = _thermal(precision)
    a, b = {}, {}
    ea = oracle_run(orc, deck, packed, 8, out_state=a)
    eb = oracle_run(orc, deck, packed, 8, out_state=b)
    assert np.array_equal(ea, eb)
    assert np.array_equal(a["particles"], b["particles"])
    assert np.array_equal(a["fields"], b["fields"])


def test_fp64_oracle_conserves_charge(orc):
    deck, packed = _thermal(8, n=8, ppc=16, steps=12)
    p = deck.derived()
    nx = ny = nz = deck.nx
    dxyz = (float(p["dx"]), float(p["dy"]), float(p["dz"]))
    eps0 = float(p["eps"])

    def residual(state):
        part = L.unpack_particles(state["particles"], deck.num_particles, deck.R, deck.vl)
        rho = od.charge_density(part, nx, ny, nz, float(p["qsp"]), *dxyz)
        return od.gauss_residual(state["fields"], rho, nx, ny, nz, *dxyz, eps0=eps0), np.abs(rho).max()

    st = {"particles": packed, "fields": np.zeros((deck.num_cells, 9))}
    r0, rho_max = residual(st)
    worst = 0.0
    crossed = 0
    for _ in range(12):
        prev = L.unpack_particles(st["particles"], deck.num_particles, deck.R, deck.vl)["cell"]
        nxt = {}
        oracle_run(orc, deck, st["particles"], 1, fields_init=st["fields"], out_state=nxt)
        crossed += int(np.count_nonzero(
            L.unpack_particles(nxt["particles"], deck.num_particles, deck.R, deck.vl)["cell"] != prev))
        st = nxt
        r, _ = residual(st)
        worst = max(worst, float(np.abs(r - r0).max()) / rho_max)
    assert crossed > deck.num_particles // 10  # the plasma really crosses cells
    assert worst < 1e-12, worst


def test_omp_push_matches_serial_push(orc):
    deck, packed = _thermal(4, n=8, ppc=16)
    p = deck.derived()
    g = orc.grid(deck.nx, deck.ny, deck.nz)
    rng = np.random.default_rng(3)
    fields = L.pack_cells(rng.normal(0, 0.05, (deck.num_cells, 9)).astype(np.float32), np.float32)
    interp = np.zeros(L.cell_array_bytes(deck.num_cells, 18, np.float32) // 4, np.float32)
    orc.load_interpolator(fields, interp, g)
    args = (interp, p["qdt_2mc"], p["cdt_dx"], p["cdt_dy"], p["cdt_dz"], p["qsp"])
    serial, omp = packed.copy(), packed.copy()
    acc_s = np.zeros((deck.num_cells, 3, 4), np.float32)
    acc_o = np.zeros_like(acc_s)
    acc_abs = np.zeros(acc_s.shape, np.float32)
    acc_cnt = np.zeros(acc_s.shape, np.int32)
    orc.push(serial, deck.num_particles, deck.vl, *args, acc_s, g, acc_abs=acc_abs, acc_count=acc_cnt)
    orc.push_omp(omp, deck.num_particles, deck.vl, *args, acc_o, g, 4)
    assert np.array_equal(serial, omp)
    bound = reorder_bound(acc_abs, acc_cnt, np.finfo(np.float32).eps)
    assert np.all(np.abs(acc_o.astype(np.float64) - acc_s) <= bound + 1e-30)


@pytest.mark.parametrize("precision", [4, 8])
def test_oracle_thermal_loader_matches_host_restatement(orc, precision):
    """The oracle's OpenMP thermal loader (the CPU baseline's input at full
    size) gives the host restatement's particles: offsets, weights and cells
    bit for bit, momenta within one rounding of the libm calls."""
    d = decks.thermal(n=10, ppc=7, precision=precision, seed=99)
    want = decks.thermal_particles(d)
    got = L.unpack_particles(orc.thermal_particles(d), d.num_particles, d.R, d.vl)
    for k in ("x", "y", "z", "w", "cell"):
        assert np.array_equal(got[k], want[k]), k
    eps = np.finfo(d.R).eps
    for k in ("ux", "uy", "uz"):
        assert np.all(np.abs(got[k] - want[k]) <= 2 * eps * np.abs(want[k])), k
