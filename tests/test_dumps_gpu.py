"""Particle and field dumps: the reference's text formats (dump_particles,
src/helpers.h:31-61; dump_fields, src/fields.h:318-350; the per-step headers
of example/example.cpp:131-132, 273-277), written from asynchronous copies of
device-computed values, against the same text formatted on the host from the
downloaded state with the reference's arithmetic."""
import io

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def _ref_particle_line(p, R, dx, nx, ny):
    from cabanapic_gb300 import layout as L
    ix, _, _ = L.rank_to_index(p["cell"].astype(np.int64), nx, ny)
    x = (0.0 + ((ix - 1).astype(np.float64) + (p["x"].astype(np.float64) + 1.0) * 0.5) * float(dx)).astype(R)
    return "".join(f"{a:e}  {b:e} " for a, b in zip(x.astype(np.float64), p["ux"].astype(np.float64))) + "\n"


def _ref_field_block(fm, R, dx, nx, ny):
    out = []
    for i in range(1, nx + 1):
        x = R(0.0 + (i - 0.5) * float(dx))
        ii = i + (nx + 2) * (1 + (ny + 2) * 1)
        out.append(f"{float(x):e} {float(fm[ii, 0]):e}\n")
    return "".join(out) + "\n\n"


@pytest.mark.parametrize("precision", [4, 8])
def test_time_loop_dumps_match_reference_format(precision):
    from cabanapic_gb300 import decks
    from cabanapic_gb300.simulation import Simulation
    deck = decks.two_stream_em(precision=precision, num_steps=4)
    R = deck.R
    p = deck.derived()
    fp_p, fp_f = io.StringIO(), io.StringIO()
    sim = Simulation(deck, particle_dump=fp_p, field_dump=fp_f)
    expect_p = ["#step=0\n0 " + _ref_particle_line(sim.particles.download(), R, p["dx"], deck.nx, deck.ny)]
    expect_f = []
    for k in range(1, 4):
        sim.step()
        torch.cuda.synchronize()
        t = float(R(R(k) * p["dt"]))
        expect_p.append(f"#step={k}\n{t:e} " + _ref_particle_line(sim.particles.download(), R, p["dx"],
                                                                    deck.nx, deck.ny))
        expect_f.append(f"#step={k}\n" + _ref_field_block(sim.fields.get_members(), R, p["dx"], deck.nx,
                                                           deck.ny))
    sim.flush_dumps()
    assert fp_p.getvalue() == "".join(expect_p)
    assert fp_f.getvalue() == "".join(expect_f)


def test_cpp_shim_dumps_agree_with_python(tmp_path):
    """minipic (the C++ shim's dump_particles / dump_fields, printed with
    fprintf like the reference) and the Python time loop write the same files:
    byte-identical at t = 0, the same structure and values to round-off
    afterwards (the deposit's atomics reorder sums between runs)."""
    import subprocess
    from cabanapic_gb300 import build, decks
    from cabanapic_gb300.simulation import Simulation
    exe = build.MINIPIC_F64
    fp, ff = tmp_path / "p.txt", tmp_path / "f.txt"
    subprocess.run([exe, "3", str(tmp_path / "e.txt"), str(fp), str(ff)], check=True, timeout=120)
    deck = decks.two_stream_em(precision=8, num_steps=3)
    sp, sf = io.StringIO(), io.StringIO()
    sim = Simulation(deck, particle_dump=sp, field_dump=sf)
    sim.run(3)
    sim.flush_dumps()
    cpp_p, py_p = fp.read_text().split("\n"), sp.getvalue().split("\n")
    cpp_f, py_f = ff.read_text(), sf.getvalue()
    assert cpp_p[:2] == py_p[:2]
    assert len(cpp_p) == len(py_p) and [l for l in cpp_p if l.startswith("#")] == [l for l in py_p if l.startswith("#")]
    a = np.array([float(t) for l in cpp_p if l and not l.startswith("#") for t in l.split()])
    b = np.array([float(t) for l in py_p if l and not l.startswith("#") for t in l.split()])
    np.testing.assert_allclose(a, b, rtol=1e-9, atol=1e-12)
    fa = np.array([float(t) for l in cpp_f.split("\n") if l and not l.startswith("#") for t in l.split()])
    fb = np.array([float(t) for l in py_f.split("\n") if l and not l.startswith("#") for t in l.split()])
    assert cpp_f.count("#step=") == 3 and fa.shape == fb.shape
    np.testing.assert_allclose(fa, fb, rtol=1e-6, atol=1e-15)
