"""CPU-side checks of the C-ABI library: it loads, exports every entry point
that include/cpic/capi.h declares, and rejects bad arguments before any CUDA
call (so these run without a GPU)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "cpic", "capi.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cpic_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from cabanapic_gb300 import build, capi
    build.build()
    return capi.load()


def test_header_declares_the_expected_entry_points():
    names = _declared()
    for must in ("cpic_push", "cpic_load_interpolator", "cpic_unload_accumulator",
                 "cpic_clear_accumulator", "cpic_advance_b", "cpic_advance_e",
                 "cpic_field_energies", "cpic_sort_particles", "cpic_status_read"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in _declared() if not hasattr(lib.dll, n)]
    assert not missing, missing


def test_binding_covers_the_header(lib):
    from cabanapic_gb300 import capi
    assert set(_declared()) <= set(capi.exported_symbols())


def test_version_and_strerror(lib):
    assert lib.dll.cpic_version() >= 1
    assert lib.dll.cpic_strerror(-2).decode().startswith("unsupported")
    assert lib.dll.cpic_strerror(12345).decode() == "unknown cpic error"


def _prm(**kw):
    from cabanapic_gb300 import capi
    d = dict(qdt_2mc=-0.01, cdt_dx=0.5, cdt_dy=0.5, cdt_dz=0.5, qsp=-1.0, precision=4,
             particle_vl=32, flags=0, reserved=0)
    d.update(kw)
    return capi.CpicPushParams(**d)


def test_push_argument_validation(lib):
    from cabanapic_gb300 import capi
    push = lib.raw("cpic_push")
    g = capi.make_grid(4, 4, 4)
    status = C.c_int32(0)
    dummy = C.c_void_p(64)  # never dereferenced: validation fails first
    assert push(dummy, 10, dummy, dummy, None, C.byref(_prm()), C.byref(status), None) == capi.CPIC_EINVAL
    assert push(dummy, 10, dummy, dummy, C.byref(g), None, C.byref(status), None) == capi.CPIC_EINVAL
    assert push(dummy, 10, dummy, dummy, C.byref(g), C.byref(_prm(precision=2)), C.byref(status), None) == capi.CPIC_EINVAL
    assert push(dummy, 10, dummy, dummy, C.byref(g), C.byref(_prm(particle_vl=8)), C.byref(status), None) == capi.CPIC_EINVAL
    assert push(dummy, 10, dummy, dummy, C.byref(g), C.byref(_prm(flags=32)), C.byref(status), None) == capi.CPIC_EINVAL
    # LayoutLeft accumulators hold real_t values, not the FP64 rows of an FP32 push
    left64 = capi.CPIC_PUSH_ACC_LAYOUT_LEFT | capi.CPIC_PUSH_ACC_F64
    assert push(dummy, 10, dummy, dummy, C.byref(g), C.byref(_prm(flags=left64)), C.byref(status), None) == capi.CPIC_EINVAL
    assert push(None, 10, dummy, dummy, C.byref(g), C.byref(_prm()), C.byref(status), None) == capi.CPIC_EINVAL
    assert push(dummy, -1, dummy, dummy, C.byref(g), C.byref(_prm()), C.byref(status), None) == capi.CPIC_EINVAL
    # empty particle list: nothing to do, no device access
    assert push(None, 0, None, None, C.byref(g), C.byref(_prm()), C.byref(status), None) == capi.CPIC_OK
    refl = capi.make_grid(4, 4, 4, 1, capi.CPIC_REFLECT)
    assert push(dummy, 10, dummy, dummy, C.byref(refl), C.byref(_prm()), C.byref(status), None) == capi.CPIC_EUNSUPPORTED
    ng2 = capi.make_grid(4, 4, 4, 2)
    assert push(dummy, 10, dummy, dummy, C.byref(ng2), C.byref(_prm()), C.byref(status), None) == capi.CPIC_EUNSUPPORTED
    bad = capi.make_grid(0, 4, 4)
    assert push(dummy, 10, dummy, dummy, C.byref(bad), C.byref(_prm()), C.byref(status), None) == capi.CPIC_EINVAL
    # misaligned accumulator (vector reductions need 16-byte alignment)
    assert push(dummy, 10, dummy, C.c_void_p(68), C.byref(g), C.byref(_prm()), C.byref(status), None) == capi.CPIC_EINVAL


def test_adjoint_push_argument_validation(lib):
    from cabanapic_gb300 import capi
    f = lib.raw("cpic_adjoint_push")
    g = capi.make_grid(4, 4, 4)
    status = C.c_int32(0)
    d = C.c_void_p(64)  # never dereferenced: validation fails first
    rows = _prm(precision=8, flags=capi.CPIC_ADJ_INTERP_ROWS)
    # the push's accumulator flags have no adjoint
    assert f(d, 10, d, d, d, d, C.byref(g), C.byref(_prm(flags=capi.CPIC_PUSH_ACC_F64)), C.byref(status), None) == capi.CPIC_EINVAL
    assert f(d, 10, d, d, d, None, C.byref(g), C.byref(rows), C.byref(status), None) == capi.CPIC_EINVAL
    # interpolator-adjoint rows must start on a 16-byte boundary
    assert f(d, 10, d, d, d, C.c_void_p(72), C.byref(g), C.byref(rows), C.byref(status), None) == capi.CPIC_EINVAL
    assert f(None, 0, None, None, None, None, C.byref(g), C.byref(rows), C.byref(status), None) == capi.CPIC_OK
    assert capi.CPIC_ADJ_INTERP_ROW >= 18 and capi.CPIC_ADJ_INTERP_ROW * 4 % 16 == 0
    rows_load = lib.raw("cpic_adjoint_load_interpolator_rows")
    assert rows_load(C.c_void_p(72), d, C.byref(g), 4, None) == capi.CPIC_EINVAL
    assert rows_load(None, d, C.byref(g), 4, None) == capi.CPIC_EINVAL
    unload_adj = lib.raw("cpic_adjoint_unload_accumulator")
    assert unload_adj(d, C.c_void_p(72), C.byref(g), 1.0, 1.0, 1.0, 1.0, 4, None) == capi.CPIC_EINVAL


def test_look_ahead_sort_argument_validation(lib):
    from cabanapic_gb300 import capi
    f = lib.raw("cpic_sort_particles_ahead_into")
    g = capi.make_grid(4, 4, 4)
    a, b, sc = C.c_void_p(4096), C.c_void_p(1 << 20), C.c_void_p(1 << 24)
    ok = _prm()
    assert f(a, b, 10, None, C.byref(ok), 5, sc, 1 << 20, None) == capi.CPIC_EINVAL
    assert f(a, b, 10, C.byref(g), None, 5, sc, 1 << 20, None) == capi.CPIC_EINVAL
    assert f(a, b, 10, C.byref(g), C.byref(ok), -1, sc, 1 << 20, None) == capi.CPIC_EINVAL
    assert f(a, b, 10, C.byref(g), C.byref(_prm(cdt_dx=float("nan"))), 5, sc, 1 << 20, None) == capi.CPIC_EINVAL
    assert f(a, b, 10, C.byref(g), C.byref(_prm(particle_vl=8)), 5, sc, 1 << 20, None) == capi.CPIC_EINVAL
    assert f(a, a, 10, C.byref(g), C.byref(ok), 5, sc, 1 << 20, None) == capi.CPIC_EINVAL  # overlapping
    assert f(a, b, 10, C.byref(g), C.byref(ok), 5, C.c_void_p((1 << 24) + 16), 1 << 20, None) == capi.CPIC_EINVAL
    # scratch smaller than cpic_sort_into_scratch_bytes
    assert f(a, b, 10, C.byref(g), C.byref(ok), 5, sc, 16, None) == capi.CPIC_ESCRATCH
    assert f(None, None, 0, C.byref(g), C.byref(ok), 5, None, 0, None) == capi.CPIC_OK
    refl = capi.make_grid(4, 4, 4, 1, capi.CPIC_REFLECT)
    assert f(a, b, 10, C.byref(refl), C.byref(ok), 5, sc, 1 << 20, None) == capi.CPIC_EUNSUPPORTED


def test_push_into_argument_validation(lib):
    from cabanapic_gb300 import capi
    f = lib.raw("cpic_push_into")
    g = capi.make_grid(4, 4, 4)
    status = C.c_int32(0)
    d, e = C.c_void_p(64), C.c_void_p(128)
    assert f(d, e, 10, d, d, C.byref(g), C.byref(_prm(flags=capi.CPIC_PUSH_STREAMING)), C.byref(status), None) == capi.CPIC_EUNSUPPORTED
    assert f(d, d, 10, d, d, C.byref(g), C.byref(_prm()), C.byref(status), None) == capi.CPIC_EINVAL
    # overlapping lists (10 FP32 particles take one 1 KiB block)
    assert f(C.c_void_p(4096), C.c_void_p(4096 + 512), 10, d, d, C.byref(g), C.byref(_prm()), C.byref(status), None) == capi.CPIC_EINVAL
    assert f(d, None, 10, d, d, C.byref(g), C.byref(_prm()), C.byref(status), None) == capi.CPIC_EINVAL
    assert f(d, C.c_void_p(72), 10, d, d, C.byref(g), C.byref(_prm()), C.byref(status), None) == capi.CPIC_EINVAL
    assert f(None, None, 0, None, None, C.byref(g), C.byref(_prm()), C.byref(status), None) == capi.CPIC_OK


def test_field_argument_validation(lib):
    from cabanapic_gb300 import capi
    g = capi.make_grid(4, 4, 4)
    d = C.c_void_p(64)
    assert lib.raw("cpic_load_interpolator")(None, d, C.byref(g), 4, None) == capi.CPIC_EINVAL
    assert lib.raw("cpic_load_interpolator")(d, d, C.byref(g), 3, None) == capi.CPIC_EINVAL
    assert lib.raw("cpic_advance_b")(d, 0.1, 0.1, 0.1, C.byref(capi.make_grid(4, 4, 4, 1, 0)), 4, None) == capi.CPIC_EUNSUPPORTED
    assert lib.raw("cpic_advance_e")(None, 0.1, 0.1, 0.1, C.byref(g), 0.1, 4, None) == capi.CPIC_EINVAL
    assert lib.raw("cpic_unload_accumulator")(d, None, C.byref(g), 1.0, 1.0, 1.0, 1.0, 4, None) == capi.CPIC_EINVAL
    assert lib.raw("cpic_unload_accumulator_left")(d, None, C.byref(g), 1.0, 1.0, 1.0, 1.0, 4, None) == capi.CPIC_EINVAL
    assert lib.raw("cpic_unload_accumulator_left")(d, d, C.byref(g), 1.0, 1.0, 1.0, 1.0, 2, None) == capi.CPIC_EINVAL
    assert lib.raw("cpic_field_energies")(d, C.byref(g), 4, d, d, 8, None) == capi.CPIC_ESCRATCH
    assert lib.raw("cpic_energy_scratch_bytes")() > 0


def test_sort_scratch_query(lib):
    q = lib.raw("cpic_sort_scratch_bytes")
    from cabanapic_gb300 import layout as L
    n, nc = 100000, 5000
    b = q(n, nc, 4, 32)
    assert b >= L.particle_list_bytes(n, np.float32, 32) + 4 * n + 4 * nc
    assert q(n, nc, 3, 32) == 0 and q(n, nc, 4, 7) == 0 and q(-1, nc, 4, 32) == 0


def test_no_allocation_calls_in_library_sources():
    """The library allocates nothing: scratch comes from the caller."""
    csrc = os.path.join(ROOT, "cabanapic_gb300", "csrc")
    for f in os.listdir(csrc):
        if f.endswith(".cu"):
            s = open(os.path.join(csrc, f)).read()
            assert "cudaMalloc" not in s and "cudaFree" not in s, f
