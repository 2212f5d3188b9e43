"""Seeded device particle loading (cpic_thermal_particles) against the host
restatement of the same Philox4x32-10 stream (cabanapic_gb300.decks)."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,vl", [(4, 32), (4, 16), (8, 32), (8, 16)])
def test_device_thermal_matches_host_restatement(prec, vl):
    """Offsets, weights and cells bit for bit; momenta to the rounding of the
    CUDA and libm log/cos (one rounding of a double to real_t)."""
    from cabanapic_gb300 import decks
    d = decks.thermal(n=12, ppc=48, precision=prec, vl=vl, num_steps=1, seed=(7 << 33) + 5)
    host = decks.thermal_particles(d)
    dev = decks.thermal_particles_device(d, device="cuda").download()
    for k in ("x", "y", "z", "w", "cell"):
        assert np.array_equal(dev[k], host[k]), k
    for k in ("ux", "uy", "uz"):
        a, b = dev[k].astype(np.float64), host[k].astype(np.float64)
        if prec == 4:
            ulp = np.spacing(np.abs(host[k])).astype(np.float64)
            assert np.all(np.abs(a - b) <= ulp), k
            assert np.count_nonzero(a != b) <= max(2, len(a) // 10000), k
        else:
            # the host forms cos(pi * 2u) from a rounded argument, the device
            # cospi(2u): ~1e-16 absolute apart near the zeros of the cosine
            np.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-15)


def test_device_thermal_partial_list_and_validation():
    """A list shorter than ppc x cells takes the first particles of the
    sequence; more particles than the grid holds, or a bad ppc, is rejected
    before any device work."""
    from cabanapic_gb300 import capi, decks, pic
    d = decks.thermal(n=6, ppc=16, precision=4, num_steps=1, seed=3)
    P = pic.ParticleList(1000, np.float32, 32)
    pic.thermal_particles(P, 16, 6, 6, 6, 0.05, 0.25, 3)
    got = P.download()
    ref = decks.thermal_particles(d, n_sample=1000)
    for k in ("x", "y", "z", "cell"):
        assert np.array_equal(got[k], ref[k])
    assert np.all(got["w"] == np.float32(0.25))
    f = capi.load().raw("cpic_thermal_particles")
    g = capi.make_grid(6, 6, 6)
    assert f(P.ptr, 6 ** 3 * 16 + 1, 16, C.byref(g), 0.05, 1.0, 3, 4, 32, None) == capi.CPIC_EINVAL
    assert f(P.ptr, 1000, 0, C.byref(g), 0.05, 1.0, 3, 4, 32, None) == capi.CPIC_EINVAL
    assert f(P.ptr, 1000, 16, C.byref(g), -1.0, 1.0, 3, 4, 32, None) == capi.CPIC_EINVAL


def test_simulation_loads_thermal_decks_on_the_device():
    """Simulation(particles=None) on a thermal deck fills the list on the
    device with the deck's seeded stream."""
    from cabanapic_gb300 import decks
    from cabanapic_gb300.simulation import Simulation
    d = decks.thermal(n=8, ppc=8, precision=4, num_steps=2, seed=11)
    sim = Simulation(d)
    got = sim.download_particles()
    ref = decks.thermal_particles(d)
    for k in ("x", "y", "z", "w", "cell"):
        assert np.array_equal(got[k], ref[k])
    sim.run(2)
    sim.check_status()
