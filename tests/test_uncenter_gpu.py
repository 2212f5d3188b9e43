"""uncenter_particles (the reference's t = 0 back half-step of the momenta)
on the GPU against the oracle: bit-identical (unfused arithmetic)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from support import random_state  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("real,vl", [(np.float32, 32), (np.float32, 16), (np.float64, 32)])
def test_uncenter_matches_oracle(orc, real, vl):
    from cabanapic_gb300 import pic
    st = random_state(nx=5, ny=6, nz=4, n=7001, seed=31, real=real, vl=vl)
    qdt_2mc = real(-0.037)
    ref = st["particles"].copy()
    orc.uncenter(ref, st["n"], vl, st["interp"], qdt_2mc)
    P = pic.ParticleList(st["n"], real, vl).upload(st["particles"])
    I = pic.InterpolatorArray(st["num_cells"], real)
    I.buf.copy_(torch.from_numpy(st["interp"]))
    pic.uncenter_particles(P, I, qdt_2mc, nx=st["nx"], ny=st["ny"], nz=st["nz"])
    pic.check_status()
    got = P.download_bytes()
    assert np.array_equal(got, ref)
    # only the momenta change
    a = P.download()
    assert np.array_equal(a["x"], st["host"]["x"]) and np.array_equal(a["cell"], st["host"]["cell"])
