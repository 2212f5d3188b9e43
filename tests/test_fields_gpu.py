"""Parity of the per-cell kernels against the oracle: interpolator load,
accumulator clear/unload, jf fold + ghost copy, advance_b / advance_e, and the
field energies.  The stencils are deterministic and compiled without FMA
contraction, so field values must be bit-identical."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from support import random_fields  # noqa: E402

pytestmark = pytest.mark.gpu

GRIDS = [(7, 5, 6), (1, 32, 1), (32, 1, 1), (3, 1, 9), (33, 2, 3)]


def _dev_fields(vals, nc, real):
    from cabanapic_gb300 import pic
    F = pic.FieldArray(nc, real)
    F.buf.copy_(torch.from_numpy(vals.copy()))
    return F


@pytest.mark.parametrize("real", [np.float32, np.float64])
@pytest.mark.parametrize("g", GRIDS)
def test_load_interpolator(orc, g, real):
    from cabanapic_gb300 import pic
    nx, ny, nz = g
    f, nc = random_fields(nx, ny, nz, seed=1, real=real)
    F = _dev_fields(f, nc, real)
    I = pic.InterpolatorArray(nc, real)
    pic.load_interpolator_array(F, I, nx, ny, nz, 1)
    ref = np.zeros_like(I.buf.cpu().numpy())
    orc.load_interpolator(f, ref, orc.grid(nx, ny, nz))
    assert np.array_equal(I.buf.cpu().numpy(), ref)


@pytest.mark.parametrize("real", [np.float32, np.float64])
@pytest.mark.parametrize("g", GRIDS)
def test_unload_accumulator(orc, g, real):
    from cabanapic_gb300 import pic
    nx, ny, nz = g
    f, nc = random_fields(nx, ny, nz, seed=2, real=real)
    acc = np.random.default_rng(3).standard_normal((nc, 3, 4)).astype(real)
    F = _dev_fields(f, nc, real)
    A = pic.AccumulatorArray(nc, real)
    A.set(acc)
    dx, dy, dz, dt = real(0.3), real(0.25), real(0.2), real(0.07)
    pic.unload_accumulator_array(F, A, nx, ny, nz, 1, dx, dy, dz, dt)
    ref = f.copy()
    orc.unload_accumulator(ref, acc, orc.grid(nx, ny, nz), dx, dy, dz, dt)
    assert np.array_equal(F.buf.cpu().numpy(), ref)


@pytest.mark.parametrize("real", [np.float32, np.float64])
@pytest.mark.parametrize("g", GRIDS)
def test_unload_accumulator_layout_left(g, real):
    """cpic_unload_accumulator_left reads Kokkos' LayoutLeft accumulator (the
    Kokkos-Cuda default, src/types.h:120) and writes the LayoutRight unload's
    jf bits: the same sums in the same order."""
    from cabanapic_gb300 import pic
    nx, ny, nz = g
    f, nc = random_fields(nx, ny, nz, seed=12, real=real)
    acc = np.random.default_rng(13).standard_normal((nc, 3, 4)).astype(real)
    out = []
    for layout in ("right", "left"):
        F = _dev_fields(f, nc, real)
        A = pic.AccumulatorArray(nc, real, layout=layout)
        A.set(acc)
        assert np.array_equal(A.get(), acc)
        pic.unload_accumulator_array(F, A, nx, ny, nz, 1, real(0.3), real(0.25), real(0.2), real(0.07))
        out.append(F.buf.cpu().numpy())
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("real", [np.float32, np.float64])
@pytest.mark.parametrize("g", GRIDS)
def test_advance_b(orc, g, real):
    from cabanapic_gb300 import pic
    nx, ny, nz = g
    f, nc = random_fields(nx, ny, nz, seed=4, real=real)
    F = _dev_fields(f, nc, real)
    px, py, pz = [real(v) if n > 1 else real(0) for v, n in zip((0.31, 0.27, 0.22), g)]
    pic.EMFieldSolver().advance_b(F, px, py, pz, nx, ny, nz, 1)
    ref = f.copy()
    orc.advance_b(ref, px, py, pz, orc.grid(nx, ny, nz))
    assert np.array_equal(F.buf.cpu().numpy(), ref)


@pytest.mark.parametrize("real", [np.float32, np.float64])
@pytest.mark.parametrize("g", GRIDS)
def test_advance_e(orc, g, real):
    from cabanapic_gb300 import pic
    nx, ny, nz = g
    f, nc = random_fields(nx, ny, nz, seed=5, real=real)
    F = _dev_fields(f, nc, real)
    px, py, pz = [real(v) if n > 1 else real(0) for v, n in zip((0.61, 0.57, 0.42), g)]
    dt_eps0 = real(0.037)
    pic.EMFieldSolver().advance_e(F, px, py, pz, nx, ny, nz, 1, dt_eps0)
    ref = f.copy()
    orc.advance_e(ref, px, py, pz, orc.grid(nx, ny, nz), dt_eps0)
    assert np.array_equal(F.buf.cpu().numpy(), ref)


@pytest.mark.parametrize("real", [np.float32, np.float64])
@pytest.mark.parametrize("g", GRIDS)
def test_energies(orc, g, real):
    from cabanapic_gb300 import pic
    nx, ny, nz = g
    f, nc = random_fields(nx, ny, nz, seed=6, real=real)
    F = _dev_fields(f, nc, real)
    out = pic.EMFieldSolver().energies_async(F, nx, ny, nz, 1).cpu().numpy()
    ref = orc.energies(f, orc.grid(nx, ny, nz))  # [E_real, B_real, E_double, B_double]
    assert np.allclose(out, ref[2:4], rtol=1e-12, atol=0)
    # deterministic: the same call gives the same bits
    out2 = pic.EMFieldSolver().energies_async(F, nx, ny, nz, 1).cpu().numpy()
    assert np.array_equal(out, out2)


def test_clear_and_initialize(orc):
    from cabanapic_gb300 import pic
    nc = 1000
    A = pic.AccumulatorArray(nc, np.float32)
    A.buf.fill_(3.0)
    pic.clear_accumulator_array(None, A, 8, 8, 8)
    assert float(A.buf.abs().max()) == 0.0
    I = pic.InterpolatorArray(nc, np.float32)
    I.buf.fill_(1.0)
    pic.initialize_interpolator(I)
    assert float(I.buf.abs().max()) == 0.0


@pytest.mark.parametrize("real", [np.float32, np.float64])
@pytest.mark.parametrize("fold", [True, False])
@pytest.mark.parametrize("g", [(16, 1, 1), (7, 5, 6)])
def test_es_solver(orc, g, real, fold):
    """ES_Field_Solver(_1D)::advance_e and e_energy against the oracle."""
    from cabanapic_gb300 import pic
    nx, ny, nz = g
    f, nc = random_fields(nx, ny, nz, seed=11, real=real)
    F = _dev_fields(f, nc, real)
    s = pic.ESFieldSolver1D(one_d=fold)
    cj = real(0.37)
    s.advance_e(F, 0, 0, 0, nx, ny, nz, 1, cj)
    ref = f.copy()
    orc.es_advance_e(ref, orc.grid(nx, ny, nz), cj, fold)
    assert np.array_equal(F.buf.cpu().numpy(), ref)
    e = s.e_energy(F, 0, 0, 0, nx, ny, nz, 1)
    assert abs(e / orc.es_energy(ref, orc.grid(nx, ny, nz)) - 1) < 1e-13
    s.advance_b(F, 0, 0, 0, nx, ny, nz, 1)  # a no-op in the reference
    assert np.array_equal(F.buf.cpu().numpy(), ref)
