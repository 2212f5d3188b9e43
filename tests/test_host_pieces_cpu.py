"""Host-side helpers of the overlapped host copies (Simulation.run_from_host):
the split of a particle list into runs of whole AoSoA blocks, and block-aligned
views of a list (CPU tensors stand in for device memory)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("n,vl,pieces", [(1, 32, 8), (31, 32, 8), (32, 32, 8), (1000, 32, 8), (1000, 16, 3),
                                         (134217728, 32, 8), (100, 32, 1), (64, 32, 100)])
def test_block_pieces_cover_the_list_in_whole_blocks(n, vl, pieces):
    from cabanapic_gb300.arrays import block_pieces
    runs = block_pieces(n, vl, pieces)
    assert 1 <= len(runs) <= pieces
    assert runs[0][0] == 0
    for (s0, c0), (s1, _) in zip(runs, runs[1:]):
        assert s0 + c0 == s1 and c0 % vl == 0
    assert all(s % vl == 0 and c > 0 for s, c in runs)
    assert sum(c for _, c in runs) == n


def test_particle_list_view_shares_memory_and_checks_alignment():
    from cabanapic_gb300 import layout as L
    from cabanapic_gb300.arrays import ParticleList
    n, vl = 100, 32
    P = ParticleList(n, np.float32, vl, device="cpu")
    rng = np.random.default_rng(1)
    host = {k: rng.standard_normal(n).astype(np.float32) for k in ("x", "y", "z", "ux", "uy", "uz", "w")}
    host["cell"] = rng.integers(0, 50, n).astype(np.int32)
    P.upload(host)
    v = P.view(32, 50)
    assert v.n == 50 and v.vl == vl and v.buf.data_ptr() == P.buf.data_ptr() + L.particle_block_bytes(np.float32, vl)
    got = v.download()
    for k in host:
        assert np.array_equal(got[k], host[k][32:82])
    tail = P.view(96, 4)
    assert np.array_equal(tail.download()["cell"], host["cell"][96:])
    for start, count in ((16, 10), (-32, 10), (64, 40), (0, -1)):
        with pytest.raises(ValueError):
            P.view(start, count)


def test_run_from_host_rejects_unsuitable_host_buffers():
    """Simulation.run_from_host checks its host buffers before any copy: a
    pinned uint8 tensor of the list's size in, likewise out, energies [steps, 2]."""
    from types import SimpleNamespace
    from cabanapic_gb300.simulation import Simulation
    fake = SimpleNamespace(particles=SimpleNamespace(nbytes=4096))
    ok_size = torch.zeros(4096, dtype=torch.uint8)  # not pinned (no GPU here)
    with pytest.raises(ValueError):
        Simulation.run_from_host(fake, ok_size, 3)
    with pytest.raises(ValueError):
        Simulation.run_from_host(fake, torch.zeros(1024, dtype=torch.float32), 3)
    with pytest.raises(ValueError):
        Simulation.run_from_host(fake, None, 3)
    with pytest.raises(ValueError):
        Simulation.run_from_host(fake, ok_size, 0)


@pytest.fixture(scope="module")
def lib():
    from cabanapic_gb300 import build, capi
    build.build()
    return capi.load()


def test_sorter_look_ahead_arguments(lib):
    """pic.Sorter takes look-ahead keys only double-buffered and with the grid
    and the cdt's; negative look-ahead is refused."""
    from cabanapic_gb300.arrays import ParticleList
    from cabanapic_gb300 import pic
    P = ParticleList(64, np.float32, 32, device="cpu")
    ahead = ((4, 4, 4), (0.4, 0.4, 0.4))
    with pytest.raises(ValueError):
        pic.Sorter(P, 216, double_buffer=False, steps_ahead=5, ahead=ahead)
    with pytest.raises(ValueError):
        pic.Sorter(P, 216, double_buffer=True, steps_ahead=5)
    with pytest.raises(ValueError):
        pic.Sorter(P, 216, double_buffer=True, steps_ahead=-1, ahead=ahead)
    s = pic.Sorter(P, 216, double_buffer=True, steps_ahead=5, ahead=ahead)
    assert s.steps_ahead == 5 and s._prm.precision == 4 and s._prm.particle_vl == 32
    assert abs(s._prm.cdt_dx - 0.4) < 1e-12 and s._grid.nx == 4
