"""The allocation-free energy entry point, cpic_field_energies_noalloc.

Some callers cannot allocate device memory: codes whose device memory all
belongs to their own pool or arena, language bindings with no CUDA allocator
to call, or a per-step diagnostic that must not allocate inside the time
loop.  For them the library keeps the energy reduction's scratch in a static
device array.  This test calls that entry point through the C ABI and checks
it against the existing entry point (which takes caller scratch), on two calls
in a row with different inputs, since the static array keeps the previous
call's contents.  The file name makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from support import random_fields  # noqa: E402

pytestmark = pytest.mark.gpu


def _lib():
    from cabanapic_gb300 import build, capi
    build.build()
    return capi.load()


def _existing(lib, F, grid, prec, out, scratch, stream):
    from cabanapic_gb300 import capi
    rc = lib.raw("cpic_field_energies")(F.data_ptr(), C.byref(grid), prec, out.data_ptr(),
                                        scratch.data_ptr(), scratch.numel(), stream)
    assert rc == capi.CPIC_OK


def _noalloc(lib, F, grid, prec, out, stream):
    from cabanapic_gb300 import capi
    rc = lib.raw("cpic_field_energies_noalloc")(F.data_ptr(), C.byref(grid), prec, out.data_ptr(), stream)
    assert rc == capi.CPIC_OK


@pytest.mark.parametrize("real", [np.float32, np.float64])
def test_noalloc_energies_match_the_scratch_entry_point_twice(real):
    from cabanapic_gb300 import capi
    lib = _lib()
    prec = np.dtype(real).itemsize
    stream = torch.cuda.current_stream().cuda_stream
    scratch = torch.zeros(lib.raw("cpic_energy_scratch_bytes")(), dtype=torch.uint8, device="cuda")
    # two different inputs, one call each, back to back
    cases = [((37, 29, 21), 11, 1.0), ((64, 8, 3), 12, 3.5)]
    for (nx, ny, nz), seed, scale in cases:
        vals, _ = random_fields(nx, ny, nz, seed=seed, real=real, scale=scale)
        F = torch.from_numpy(vals).cuda()
        grid = capi.make_grid(nx, ny, nz)
        want = torch.zeros(2, dtype=torch.float64, device="cuda")
        got = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
        _existing(lib, F, grid, prec, want, scratch, stream)
        _noalloc(lib, F, grid, prec, got, stream)
        torch.cuda.synchronize()
        w, g = want.cpu().numpy(), got.cpu().numpy()
        assert np.all(w > 0)
        # the same kernel, launch shape and reduction order: equal bit for bit
        np.testing.assert_array_equal(g, w)


def test_noalloc_rejects_grids_beyond_the_limits():
    from cabanapic_gb300 import capi
    lib = _lib()
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    F = torch.zeros(64, dtype=torch.float32, device="cuda")
    fn = lib.raw("cpic_field_energies_noalloc")
    too_big = capi.make_grid(1 << 21, 1, 1)
    assert fn(F.data_ptr(), C.byref(too_big), 4, out.data_ptr(), None) == capi.CPIC_EINVAL
    assert fn(F.data_ptr(), C.byref(capi.make_grid(4, 4, 4)), 3, out.data_ptr(), None) == capi.CPIC_EINVAL
    assert fn(None, C.byref(capi.make_grid(4, 4, 4)), 4, out.data_ptr(), None) == capi.CPIC_EINVAL
