"""ctypes binding of libcpic.so (include/cpic/capi.h).

The library must have been built (cabanapic_gb300/build.py, or
__graft_entry__.build()); there is no fallback implementation: loading fails
loudly when the shared library is missing.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

CPIC_OK = 0
CPIC_EINVAL = -1
CPIC_EUNSUPPORTED = -2
CPIC_ECUDA = -3
CPIC_ESCRATCH = -4

CPIC_STATUS_CELL_RANGE = 1
CPIC_STATUS_MOVER_CAP = 2
CPIC_STATUS_NONFINITE = 4
CPIC_STATUS_PIPELINE = 8

CPIC_REFLECT = 0
CPIC_PERIODIC = 1
CPIC_FLOAT = 4
CPIC_DOUBLE = 8
CPIC_PUSH_TRUE_SQRT = 1
CPIC_PUSH_EXACT = 2
CPIC_PUSH_STREAMING = 4
CPIC_PUSH_ACC_F64 = 8
CPIC_PUSH_ACC_LAYOUT_LEFT = 16
CPIC_ADJ_INTERP_ROWS = 32
CPIC_ADJ_INTERP_ROW = 20

_vp = C.c_void_p
_i64 = C.c_int64
_i32 = C.c_int32
_f64 = C.c_double
_sz = C.c_size_t


class CpicGrid(C.Structure):
    _fields_ = [("nx", _i64), ("ny", _i64), ("nz", _i64), ("num_ghosts", _i64),
                ("boundary", _i32), ("reserved", _i32)]


class CpicPushParams(C.Structure):
    _fields_ = [("qdt_2mc", _f64), ("cdt_dx", _f64), ("cdt_dy", _f64), ("cdt_dz", _f64),
                ("qsp", _f64), ("precision", _i32), ("particle_vl", _i32), ("flags", _i32),
                ("reserved", _i32)]


class CpicError(RuntimeError):
    """A C-ABI call returned a negative code."""

    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed: {msg} ({code})")
        self.code = code


class CpicDeviceError(RuntimeError):
    """The device status word reported a problem found inside a kernel."""

    def __init__(self, bits: int):
        names = []
        if bits & CPIC_STATUS_CELL_RANGE:
            names.append("particle cell index outside the grid")
        if bits & CPIC_STATUS_MOVER_CAP:
            names.append("move_p streak cap reached")
        if bits & CPIC_STATUS_NONFINITE:
            names.append("non-finite particle displacement")
        if bits & CPIC_STATUS_PIPELINE:
            names.append("a bounded wait in the tiled push gave up")
        super().__init__("device status %#x: %s" % (bits, "; ".join(names) or "unknown"))
        self.bits = bits


# name -> (restype, argtypes)
_SIGS = {
    "cpic_version": (_i32, []),
    "cpic_strerror": (C.c_char_p, [_i32]),
    "cpic_push": (_i32, [_vp, _i64, _vp, _vp, C.POINTER(CpicGrid), C.POINTER(CpicPushParams), _vp, _vp]),
    "cpic_load_interpolator": (_i32, [_vp, _vp, C.POINTER(CpicGrid), _i32, _vp]),
    "cpic_initialize_interpolator": (_i32, [_vp, _i64, _i32, _vp]),
    "cpic_clear_accumulator": (_i32, [_vp, _i64, _i32, _vp]),
    "cpic_unload_accumulator": (_i32, [_vp, _vp, C.POINTER(CpicGrid), _f64, _f64, _f64, _f64, _i32, _vp]),
    "cpic_advance_b": (_i32, [_vp, _f64, _f64, _f64, C.POINTER(CpicGrid), _i32, _vp]),
    "cpic_advance_e": (_i32, [_vp, _f64, _f64, _f64, C.POINTER(CpicGrid), _f64, _i32, _vp]),
    "cpic_energy_scratch_bytes": (_sz, []),
    "cpic_field_energies": (_i32, [_vp, C.POINTER(CpicGrid), _i32, _vp, _vp, _sz, _vp]),
    "cpic_field_energies_noalloc": (_i32, [_vp, C.POINTER(CpicGrid), _i32, _vp, _vp]),
    "cpic_sort_scratch_bytes": (_sz, [_i64, _i64, _i32, _i32]),
    "cpic_sort_particles": (_i32, [_vp, _i64, _i64, _i32, _i32, _vp, _sz, _vp]),
    "cpic_charge_density": (_i32, [_vp, _i64, C.POINTER(CpicGrid), _i32, _i32, _f64, _f64, _f64, _f64,
                                   _vp, _vp, _vp]),
    "cpic_diag_scratch_bytes": (_sz, []),
    "cpic_gauss_residual": (_i32, [_vp, _vp, _vp, _f64, _f64, _f64, _f64, C.POINTER(CpicGrid), _i32,
                                   _vp, _vp, _vp, _sz, _vp]),
    "cpic_kinetic_energy": (_i32, [_vp, _i64, _i32, _i32, _f64, _vp, _vp, _sz, _vp]),
    "cpic_adjoint_push": (_i32, [_vp, _i64, _vp, _vp, _vp, _vp, C.POINTER(CpicGrid),
                                 C.POINTER(CpicPushParams), _vp, _vp]),
    "cpic_adjoint_advance_b": (_i32, [_vp, _f64, _f64, _f64, C.POINTER(CpicGrid), _i32, _vp]),
    "cpic_adjoint_advance_e": (_i32, [_vp, _f64, _f64, _f64, C.POINTER(CpicGrid), _f64, _i32, _vp]),
    "cpic_adjoint_unload_accumulator": (_i32, [_vp, _vp, C.POINTER(CpicGrid), _f64, _f64, _f64, _f64,
                                               _i32, _vp]),
    "cpic_adjoint_load_interpolator": (_i32, [_vp, _vp, C.POINTER(CpicGrid), _i32, _vp]),
    "cpic_adjoint_load_interpolator_rows": (_i32, [_vp, _vp, C.POINTER(CpicGrid), _i32, _vp]),
    "cpic_uncenter_particles": (_i32, [_vp, _i64, _vp, _f64, C.POINTER(CpicGrid), _i32, _i32, _vp, _vp]),
    "cpic_es_advance_e": (_i32, [_vp, C.POINTER(CpicGrid), _f64, _i32, _i32, _vp]),
    "cpic_es_e_energy": (_i32, [_vp, C.POINTER(CpicGrid), _i32, _vp, _vp, _sz, _vp]),
    "cpic_particle_dump_values": (_i32, [_vp, _i64, _i32, C.POINTER(CpicGrid), _i32, _f64, _f64, _vp, _vp]),
    "cpic_field_dump_values": (_i32, [_vp, C.POINTER(CpicGrid), _i32, _f64, _f64, _vp, _vp]),
    "cpic_sort_into_scratch_bytes": (_sz, [_i64, _i64, _i32, _i32]),
    "cpic_sort_particles_into": (_i32, [_vp, _vp, _i64, _i64, _i32, _i32, _vp, _sz, _vp]),
    "cpic_sort_particles_ahead_into": (_i32, [_vp, _vp, _i64, C.POINTER(CpicGrid), C.POINTER(CpicPushParams),
                                               _i32, _vp, _sz, _vp]),
    "cpic_unload_accumulator_f64": (_i32, [_vp, _vp, C.POINTER(CpicGrid), _f64, _f64, _f64, _f64, _i32, _vp]),
    "cpic_unload_accumulator_left": (_i32, [_vp, _vp, C.POINTER(CpicGrid), _f64, _f64, _f64, _f64, _i32, _vp]),
    "cpic_thermal_particles": (_i32, [_vp, _i64, _i32, C.POINTER(CpicGrid), _f64, _f64, C.c_uint64, _i32,
                                      _i32, _vp]),
    "cpic_selftest_bounded_wait": (_i32, [_i64, _vp, _vp]),
    "cpic_push_into": (_i32, [_vp, _vp, _i64, _vp, _vp, C.POINTER(CpicGrid), C.POINTER(CpicPushParams), _vp,
                              _vp]),
    "cpic_status_clear": (_i32, [_vp, _vp]),
    "cpic_status_read": (_i32, [_vp, _vp, C.POINTER(_i32)]),
}


def exported_symbols():
    return list(_SIGS)


class Lib:
    def __init__(self, path: str):
        self.path = path
        self.dll = C.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(self.dll, name)
            fn.restype = res
            fn.argtypes = args

    def call(self, name: str, *args) -> int:
        rc = getattr(self.dll, name)(*args)
        if rc < 0:
            msg = self.dll.cpic_strerror(rc).decode()
            raise CpicError(name, rc, msg)
        return rc

    def raw(self, name: str):
        return getattr(self.dll, name)


_LIB = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> Lib:
    """Loads libcpic.so; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        path = _build.LIB
        if not os.path.exists(path):
            if build_if_missing:
                _build.build()
            else:
                raise ImportError(
                    f"libcpic.so not found at {path}: build it first "
                    "(python -c 'import __graft_entry__ as g; g.build()')")
        _LIB = Lib(path)
    return _LIB


def make_grid(nx, ny, nz, num_ghosts=1, boundary=CPIC_PERIODIC) -> CpicGrid:
    return CpicGrid(int(nx), int(ny), int(nz), int(num_ghosts), int(boundary), 0)
