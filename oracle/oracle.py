"""ctypes loader for the CPU oracle library (test infrastructure only)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_c_p = C.c_void_p
_i64 = C.c_int64
_i32 = C.c_int32
_f32 = C.c_float
_f64 = C.c_double


class OrcGrid(C.Structure):
    _fields_ = [("nx", _i64), ("ny", _i64), ("nz", _i64), ("ng", _i64)]


def _ptr(a) -> int:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data
    return int(a)


class Oracle:
    def __init__(self, path: str):
        self.lib = lib = C.CDLL(path)
        gp = C.POINTER(OrcGrid)
        for suf, real in (("f32", _f32), ("f64", _f64)):
            args = [_c_p, _i64, _i32, _c_p, real, real, real, real, real, _c_p, _c_p, _c_p, gp]
            if suf == "f64":
                args.append(_i32)
            args.append(_c_p)
            getattr(lib, f"orc_push_{suf}").argtypes = args
            getattr(lib, f"orc_push_omp_{suf}").argtypes = [
                _c_p, _i64, _i32, _c_p, real, real, real, real, real, _c_p, gp, _i32]
            getattr(lib, f"orc_load_interpolator_{suf}").argtypes = [_c_p, _c_p, gp]
            getattr(lib, f"orc_unload_accumulator_{suf}").argtypes = [_c_p, _c_p, gp, real, real, real, real]
            getattr(lib, f"orc_advance_b_{suf}").argtypes = [_c_p, real, real, real, gp]
            getattr(lib, f"orc_advance_e_{suf}").argtypes = [_c_p, real, real, real, gp, real]
            getattr(lib, f"orc_energies_{suf}").argtypes = [_c_p, gp, _c_p]
            getattr(lib, f"orc_current_fold_{suf}").argtypes = [_c_p, gp]
            getattr(lib, f"orc_ghost_copy_{suf}").argtypes = [_c_p, gp, _i32]
            getattr(lib, f"orc_es_advance_e_{suf}").argtypes = [_c_p, gp, real, _i32]
            getattr(lib, f"orc_es_energy_{suf}").argtypes = [_c_p, gp]
            getattr(lib, f"orc_es_energy_{suf}").restype = _f64
            getattr(lib, f"orc_default_particle_init_{suf}").argtypes = [
                _c_p, _i64, _i32, _i64, _i64, real, _i64, real, real]
        lib.orc_run_two_stream_em.argtypes = [_i32, _i32, _i32, _i32, _c_p, _c_p]
        lib.orc_uncenter_f32.argtypes = [_c_p, _i64, _i32, _c_p, _f32]
        lib.orc_uncenter_f64.argtypes = [_c_p, _i64, _i32, _c_p, _f64]
        lib.orc_num_threads.restype = _i32
        lib.orc_push_omp_sqrt_f64.argtypes = [_c_p, _i64, _i32, _c_p, _f64, _f64, _f64, _f64, _f64, _c_p, gp, _i32]
        lib.orc_thermal_particles_f32.argtypes = [_c_p, _i64, _i32, _i64, _i64, _i64, _f64, _f32, C.c_uint64]
        lib.orc_thermal_particles_f64.argtypes = [_c_p, _i64, _i32, _i64, _i64, _i64, _f64, _f64, C.c_uint64]

    @staticmethod
    def grid(nx, ny, nz, ng=1) -> OrcGrid:
        return OrcGrid(nx, ny, nz, ng)

    @staticmethod
    def _suf(dtype) -> str:
        return "f32" if np.dtype(dtype) == np.float32 else "f64"

    # ---- particle push --------------------------------------------------
    def push(self, particles: np.ndarray, n: int, vl: int, interp: np.ndarray,
             qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, acc: np.ndarray, g: OrcGrid,
             acc_abs=None, acc_count=None, literal=True) -> int:
        """Serial push; returns the number of cell-crossing particles."""
        crossers = _i64(0)
        if acc.dtype == np.float32:
            self.lib.orc_push_f32(_ptr(particles), n, vl, _ptr(interp), qdt_2mc, cdt_dx, cdt_dy,
                                  cdt_dz, qsp, _ptr(acc), _ptr(acc_abs), _ptr(acc_count),
                                  C.byref(g), C.byref(crossers))
        else:
            self.lib.orc_push_f64(_ptr(particles), n, vl, _ptr(interp), qdt_2mc, cdt_dx, cdt_dy,
                                  cdt_dz, qsp, _ptr(acc), _ptr(acc_abs), _ptr(acc_count),
                                  C.byref(g), int(literal), C.byref(crossers))
        return crossers.value

    def push_omp(self, particles, n, vl, interp, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, acc, g,
                 threads=0, literal=True) -> int:
        """Threaded push (per-thread accumulator copies, then their sum).
        literal=False (FP64 only): sqrt() for gamma instead of the
        reference's sqrtf."""
        if acc.dtype == np.float32:
            fn = self.lib.orc_push_omp_f32
        else:
            fn = self.lib.orc_push_omp_f64 if literal else self.lib.orc_push_omp_sqrt_f64
        return fn(_ptr(particles), n, vl, _ptr(interp), qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp,
                  _ptr(acc), C.byref(g), threads)

    # ---- field phase ----------------------------------------------------
    def load_interpolator(self, fields, interp, g):
        getattr(self.lib, f"orc_load_interpolator_{self._suf(fields.dtype)}")(_ptr(fields), _ptr(interp), C.byref(g))

    def unload_accumulator(self, fields, acc, g, dx, dy, dz, dt):
        getattr(self.lib, f"orc_unload_accumulator_{self._suf(fields.dtype)}")(
            _ptr(fields), _ptr(acc), C.byref(g), dx, dy, dz, dt)

    def advance_b(self, fields, px, py, pz, g):
        getattr(self.lib, f"orc_advance_b_{self._suf(fields.dtype)}")(_ptr(fields), px, py, pz, C.byref(g))

    def advance_e(self, fields, px, py, pz, g, dt_eps0):
        getattr(self.lib, f"orc_advance_e_{self._suf(fields.dtype)}")(_ptr(fields), px, py, pz, C.byref(g), dt_eps0)

    def current_fold(self, fields, g):
        getattr(self.lib, f"orc_current_fold_{self._suf(fields.dtype)}")(_ptr(fields), C.byref(g))

    def ghost_copy(self, fields, g, first_member):
        getattr(self.lib, f"orc_ghost_copy_{self._suf(fields.dtype)}")(_ptr(fields), C.byref(g), first_member)

    def energies(self, fields, g) -> np.ndarray:
        out = np.zeros(4, np.float64)
        getattr(self.lib, f"orc_energies_{self._suf(fields.dtype)}")(_ptr(fields), C.byref(g), _ptr(out))
        return out

    def default_particle_init(self, particles, n, vl, nx, ny, dxp, nppc, w, v0, dtype):
        getattr(self.lib, f"orc_default_particle_init_{self._suf(dtype)}")(
            _ptr(particles), n, vl, nx, ny, dxp, nppc, w, v0)

    def es_advance_e(self, fields, g, dt_eps0, fold=True):
        getattr(self.lib, f"orc_es_advance_e_{self._suf(fields.dtype)}")(_ptr(fields), C.byref(g), dt_eps0, int(fold))

    def es_energy(self, fields, g) -> float:
        return getattr(self.lib, f"orc_es_energy_{self._suf(fields.dtype)}")(_ptr(fields), C.byref(g))

    def uncenter(self, particles, n, vl, interp, qdt_2mc):
        getattr(self.lib, f"orc_uncenter_{self._suf(interp.dtype)}")(_ptr(particles), n, vl, _ptr(interp), qdt_2mc)

    # ---- whole runs -----------------------------------------------------
    def run_two_stream_em(self, steps: int, precision: int = 8, vl: int = 32, literal: bool = True):
        out = np.zeros((steps, 4), np.float64)
        params = np.zeros(8, np.float64)
        rc = self.lib.orc_run_two_stream_em(precision, steps, vl, int(literal), _ptr(out), _ptr(params))
        if rc != 0:
            raise RuntimeError(f"orc_run_two_stream_em failed: {rc}")
        keys = ["dt", "dx", "dy", "dz", "qdt_2mc", "we", "len_y", "py"]
        return out, dict(zip(keys, params.tolist()))

    def thermal_particles(self, deck) -> np.ndarray:
        """The thermal deck's particles (decks.thermal_particles restated in
        C with OpenMP, for large CPU baselines): packed AoSoA bytes."""
        from cabanapic_gb300 import layout as L
        R = deck.R
        n = deck.num_particles
        buf = np.empty(L.particle_list_bytes(n, R, deck.vl), np.uint8)
        getattr(self.lib, f"orc_thermal_particles_{self._suf(R)}")(
            _ptr(buf), n, deck.vl, deck.nppc, deck.nx, deck.ny, float(deck.extra.get("uth", 0.05)),
            float(deck.derived()["we"]), int(deck.extra.get("seed", 2024)) & (2 ** 64 - 1))
        return buf

    def num_threads(self) -> int:
        return self.lib.orc_num_threads()


_ORACLE = None


def load() -> Oracle:
    """Builds (if needed) and loads the oracle library."""
    global _ORACLE
    if _ORACLE is None:
        path = _build.LIB
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(_build.SRC):
            _build.build()
        _ORACLE = Oracle(path)
    return _ORACLE
