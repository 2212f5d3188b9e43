"""The reference's hot-path interface, over the C ABI.

Same names, argument order and meaning as the reference's free functions and
field solver (src/push.h, src/interpolator.h, src/accumulator.h,
src/fields.h), so a time loop reads like example/example.cpp.  Each call is
asynchronous on the current torch CUDA stream.  Argument errors raise
CpicError immediately; problems found inside kernels are collected in a device
status word and raised as CpicDeviceError by check_status().
"""
from __future__ import annotations

import ctypes as C
import enum
import os

import numpy as np
import torch

from . import capi, energies as _energies
from .arrays import AccumulatorArray, FieldArray, InterpolatorArray, ParticleList


class Boundary(enum.IntEnum):
    """Boundary, src/input/deck.h:9-12."""
    Reflect = 0
    Periodic = 1


def _stream(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


class _Status:
    """Per-device status words (one int32 each)."""

    def __init__(self):
        self.words = {}

    def get(self, device=None) -> torch.Tensor:
        dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        w = self.words.get(dev.index)
        if w is None:
            w = torch.zeros(1, dtype=torch.int32, device=dev)
            self.words[dev.index] = w
        return w


_STATUS = _Status()


def status_word(device=None) -> torch.Tensor:
    return _STATUS.get(device)


def check_status(stream=None, device=None, clear: bool = True) -> int:
    """Synchronises the stream, raises CpicDeviceError if a kernel flagged a problem."""
    lib = capi.load()
    w = _STATUS.get(device)
    out = C.c_int32(0)
    lib.call("cpic_status_read", w.data_ptr(), _stream(stream), C.byref(out))
    bits = out.value
    if clear:
        lib.call("cpic_status_clear", w.data_ptr(), _stream(stream))
    if bits:
        raise capi.CpicDeviceError(bits)
    return 0


def _grid(nx, ny, nz, ng, boundary=Boundary.Periodic):
    return capi.make_grid(nx, ny, nz, ng, int(boundary))


# ---------------------------------------------------------------- push
def push(particles: ParticleList, f0: InterpolatorArray, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp,
         a0: AccumulatorArray, g, nx, ny, nz, num_ghosts, boundary, *, true_sqrt: bool = False,
         exact: bool = False, tiles: bool = True, stream=None) -> None:
    """push() (src/push.h:7-300): Boris push, move and current deposit.

    `g` (grid_t*) is accepted and unused, as in the reference.  Adds into a0.
    exact=True selects the bit-exact variant (unfused arithmetic, IEEE
    division and sqrtf); the default uses fused multiply-adds and the hardware
    reciprocal square root (within 1e-5 relative per particle).  tiles=False
    selects the streaming kernel (no shared-memory cell windows; same
    results, slower once particles are in cell order)."""
    grid, prm = _push_args("cpic_push", particles, f0, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, a0, nx, ny,
                           nz, num_ghosts, boundary, true_sqrt, exact, tiles)
    capi.load().call("cpic_push", particles.ptr, particles.n, f0.ptr, a0.ptr, C.byref(grid), C.byref(prm),
                     _STATUS.get().data_ptr(), _stream(stream))


def push_into(particles: ParticleList, out, f0: InterpolatorArray, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp,
              a0: AccumulatorArray, g, nx, ny, nz, num_ghosts, boundary, *, true_sqrt: bool = False,
              exact: bool = False, stream=None) -> None:
    """push() out of place (cpic_push_into): particle p of `particles` (left
    unchanged) is pushed into slot p of `out` (a ParticleList or a device
    buffer of the same size), every member written.  Tiled kernel."""
    grid, prm = _push_args("cpic_push_into", particles, f0, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, a0, nx, ny,
                           nz, num_ghosts, boundary, true_sqrt, exact, True)
    dst = out.ptr if isinstance(out, ParticleList) else out.data_ptr()
    capi.load().call("cpic_push_into", particles.ptr, dst, particles.n, f0.ptr, a0.ptr, C.byref(grid),
                     C.byref(prm), _STATUS.get().data_ptr(), _stream(stream))


def _push_args(fn, particles, f0, qdt_2mc, cdt_dx, cdt_dy, cdt_dz, qsp, a0, nx, ny, nz, num_ghosts,
               boundary, true_sqrt, exact, tiles):
    # an FP64 accumulator with FP32 particles: the compensated per-cell current sum
    acc_f64 = particles.precision == capi.CPIC_FLOAT and a0.precision == capi.CPIC_DOUBLE
    left = getattr(a0, "layout", "right") == "left"
    flags = ((capi.CPIC_PUSH_TRUE_SQRT if true_sqrt else 0) | (capi.CPIC_PUSH_EXACT if exact else 0)
             | (0 if tiles else capi.CPIC_PUSH_STREAMING) | (capi.CPIC_PUSH_ACC_F64 if acc_f64 else 0)
             | (capi.CPIC_PUSH_ACC_LAYOUT_LEFT if left else 0))
    prm = capi.CpicPushParams(float(qdt_2mc), float(cdt_dx), float(cdt_dy), float(cdt_dz),
                              float(qsp), particles.precision, particles.vl, flags, 0)
    if f0.precision != particles.precision or (a0.precision != particles.precision and not acc_f64):
        raise capi.CpicError(fn, capi.CPIC_EINVAL, "mixed real_t precisions")
    grid = _grid(nx, ny, nz, num_ghosts, boundary)
    if f0.num_cells < grid_cells(nx, ny, nz, num_ghosts) or a0.num_cells < grid_cells(nx, ny, nz, num_ghosts):
        raise capi.CpicError(fn, capi.CPIC_EINVAL, "cell arrays smaller than the grid")
    return grid, prm


def thermal_particles(particles: ParticleList, ppc: int, nx, ny, nz, uth: float, weight: float,
                      seed: int, *, stream=None) -> None:
    """Seeded thermal plasma written on the device (cpic_thermal_particles):
    ppc particles per interior cell in VOXEL order, offsets uniform in
    [-1, 1), Maxwellian momenta of width uth, weight `weight`; particle p
    draws from Philox4x32-10 counters (p, 0), (p, 1) under key `seed`."""
    capi.load().call("cpic_thermal_particles", particles.ptr, particles.n, int(ppc),
                     C.byref(_grid(nx, ny, nz, 1)), float(uth), float(weight), int(seed) & (2 ** 64 - 1),
                     particles.precision, particles.vl, _stream(stream))


def grid_cells(nx, ny, nz, ng=1) -> int:
    return (nx + 2 * ng) * (ny + 2 * ng) * (nz + 2 * ng)


def uncenter_particles(particles: ParticleList, f0: InterpolatorArray, qdt_2mc, *, nx, ny, nz,
                       num_ghosts=1, stream=None) -> None:
    """uncenter_particles (src/uncenter_p.h:4-105): t = 0 back half-step of u.

    The grid extents are keyword arguments (the reference reads none; they
    bound-check the cell indices here)."""
    capi.load().call("cpic_uncenter_particles", particles.ptr, particles.n, f0.ptr, float(qdt_2mc),
                     C.byref(_grid(nx, ny, nz, num_ghosts)), particles.precision, particles.vl,
                     _STATUS.get().data_ptr(), _stream(stream))


# ---------------------------------------------------------------- cells
def load_interpolator_array(fields: FieldArray, interpolators: InterpolatorArray, nx, ny, nz, ng,
                            *, boundary=Boundary.Periodic, stream=None) -> None:
    """load_interpolator_array (src/interpolator.cpp:4-124)."""
    capi.load().call("cpic_load_interpolator", fields.ptr, interpolators.ptr,
                     C.byref(_grid(nx, ny, nz, ng, boundary)), fields.precision, _stream(stream))


def initialize_interpolator(f0: InterpolatorArray, *, stream=None) -> None:
    """initialize_interpolator (src/interpolator.cpp:125-172): zero fill."""
    capi.load().call("cpic_initialize_interpolator", f0.ptr, f0.num_cells, f0.precision, _stream(stream))


def clear_accumulator_array(fields: FieldArray, accumulators: AccumulatorArray, nx, ny, nz,
                            *, stream=None) -> None:
    """clear_accumulator_array (src/accumulator.cpp:5-43)."""
    capi.load().call("cpic_clear_accumulator", accumulators.ptr, accumulators.num_cells,
                     accumulators.precision, _stream(stream))


def unload_accumulator_array(fields: FieldArray, accumulators: AccumulatorArray, nx, ny, nz, ng,
                             dx, dy, dz, dt, *, boundary=Boundary.Periodic, stream=None) -> None:
    """unload_accumulator_array (src/accumulator.cpp:45-122).  An FP64
    accumulator with FP32 fields (the compensated current sum of an FP32 push)
    is unloaded in double and rounded once; a LayoutLeft accumulator
    (AccumulatorArray(layout="left")) through cpic_unload_accumulator_left."""
    if getattr(accumulators, "layout", "right") == "left":
        fn = "cpic_unload_accumulator_left"
    elif accumulators.precision == capi.CPIC_DOUBLE and fields.precision == capi.CPIC_FLOAT:
        fn = "cpic_unload_accumulator_f64"
    else:
        fn = "cpic_unload_accumulator"
    capi.load().call(fn, fields.ptr, accumulators.ptr,
                     C.byref(_grid(nx, ny, nz, ng, boundary)), float(dx), float(dy), float(dz),
                     float(dt), fields.precision, _stream(stream))


# ---------------------------------------------------------------- fields
class EMFieldSolver:
    """Field_Solver<EM_Field_Solver> (src/fields.h:274-379, 550-720).

    The constructor zeroes the fields like Field_Solver's (fields.h:279-315).
    `boundary` is the deck's BOUNDARY_TYPE, a global in the reference."""

    def __init__(self, fields: FieldArray = None, boundary=Boundary.Periodic):
        self.boundary = Boundary(boundary)
        self._out = None
        self._scratch = None
        if fields is not None:
            self.init(fields)

    def dump_fields(self, fp, fields: FieldArray, xmin, ymin, zmin, dx, dy, dz, nx, ny, nz, ng) -> None:
        """Field_Solver::dump_fields (src/fields.h:318-350), synchronous."""
        d = FieldDump(fields, nx)
        d.enqueue(fields, xmin, dx, nx, ny, nz, ng, self.boundary)
        d.write(fp)

    def init(self, fields: FieldArray) -> None:
        fields.buf.zero_()

    def advance_b(self, fields: FieldArray, px, py, pz, nx, ny, nz, ng, *, stream=None) -> None:
        capi.load().call("cpic_advance_b", fields.ptr, float(px), float(py), float(pz),
                         C.byref(_grid(nx, ny, nz, ng, self.boundary)), fields.precision, _stream(stream))

    def advance_e(self, fields: FieldArray, px, py, pz, nx, ny, nz, ng, dt_eps0, *, stream=None) -> None:
        capi.load().call("cpic_advance_e", fields.ptr, float(px), float(py), float(pz),
                         C.byref(_grid(nx, ny, nz, ng, self.boundary)), float(dt_eps0),
                         fields.precision, _stream(stream))

    def energies_async(self, fields: FieldArray, nx, ny, nz, ng, out: torch.Tensor = None,
                       *, stream=None) -> torch.Tensor:
        """Writes [E, B] energies (double) to a device tensor without synchronising."""
        lib = capi.load()
        if self._scratch is None:
            self._scratch = torch.zeros(lib.raw("cpic_energy_scratch_bytes")(), dtype=torch.uint8,
                                        device=fields.buf.device)
        if out is None:
            if self._out is None:
                self._out = torch.zeros(2, dtype=torch.float64, device=fields.buf.device)
            out = self._out
        lib.call("cpic_field_energies", fields.ptr, C.byref(_grid(nx, ny, nz, ng, self.boundary)),
                 fields.precision, out.data_ptr(), self._scratch.data_ptr(), self._scratch.numel(),
                 _stream(stream))
        return out

    def e_energy(self, fields: FieldArray, px, py, pz, nx, ny, nz, ng, *, stream=None) -> float:
        """EM_Field_Solver::e_energy (fields.h:556-586), accumulated in double."""
        return float(self.energies_async(fields, nx, ny, nz, ng, stream=stream)[0].item())

    def b_energy(self, fields: FieldArray, px, py, pz, nx, ny, nz, ng, *, stream=None) -> float:
        """EM_Field_Solver::b_energy (fields.h:588-615), accumulated in double."""
        return float(self.energies_async(fields, nx, ny, nz, ng, stream=stream)[1].item())


class ESFieldSolver1D:
    """Field_Solver<ES_Field_Solver_1D> (src/fields.h:467-545): advance_b is a
    no-op; advance_e folds the jf ghosts and applies E -= dt_eps0 J on every
    cell; e_energy sums E^2 over every cell (ghosts included), in double.
    one_d=False gives ES_Field_Solver (src/fields.h:382-464, no fold)."""

    def __init__(self, fields: FieldArray = None, boundary=Boundary.Periodic, one_d: bool = True):
        self.boundary = Boundary(boundary)
        self.one_d = bool(one_d)
        self._scratch = None
        if fields is not None:
            fields.buf.zero_()

    def advance_b(self, fields, px, py, pz, nx, ny, nz, ng, *, stream=None) -> None:
        return None

    def advance_e(self, fields: FieldArray, px, py, pz, nx, ny, nz, ng, dt_eps0, *, stream=None) -> None:
        capi.load().call("cpic_es_advance_e", fields.ptr, C.byref(_grid(nx, ny, nz, ng, self.boundary)),
                         float(dt_eps0), int(self.one_d), fields.precision, _stream(stream))

    def e_energy(self, fields: FieldArray, px, py, pz, nx, ny, nz, ng, *, stream=None) -> float:
        lib = capi.load()
        if self._scratch is None:
            self._scratch = torch.zeros(lib.raw("cpic_energy_scratch_bytes")(), dtype=torch.uint8,
                                        device=fields.buf.device)
        out = torch.zeros(2, dtype=torch.float64, device=fields.buf.device)
        lib.call("cpic_es_e_energy", fields.ptr, C.byref(_grid(nx, ny, nz, ng, self.boundary)),
                 fields.precision, out.data_ptr(), self._scratch.data_ptr(), self._scratch.numel(),
                 _stream(stream))
        return float(out[0].item())


def dump_energies(field_solver, fields: FieldArray, step, time, px, py, pz, nx, ny,
                  nz, ng, path: str = "energies.txt", echo: bool = True) -> tuple:
    """dump_energies (src/fields.h:722-763): appends the `step time E B` line
    to `path` in std::ostream format (truncating the file at step 0) and, as
    the reference does, prints the printf("%d %f %e %e") line to stdout
    (echo=False leaves stdout alone).  Returns (E, B).  With an ES solver
    (ESFieldSolver1D, the reference's ES_FIELD_SOLVER build) there is no B:
    the line is `step time E`, the stdout line printf("%d %f %e"), and B is
    returned as None."""
    if isinstance(field_solver, ESFieldSolver1D):
        e, b = field_solver.e_energy(fields, px, py, pz, nx, ny, nz, ng), None
    else:
        e, b = field_solver.energies_async(fields, nx, ny, nz, ng).cpu().tolist()
    mode = "w" if step == 0 else "a"
    with open(path, mode) as fh:
        fh.write(_energies.energy_line(step, time, e, b) + "\n")
    if echo:
        print(_energies.stdout_line(step, time, e, b), flush=True)
    return e, b


# ---------------------------------------------------------------- dumps
def _fmt_pairs(vals: np.ndarray, sep: str, end: str) -> str:
    """C printf "%e" of each value (Python's %e is the same format), pairs
    joined as the reference's fprintf calls write them."""
    v = vals.astype(np.float64).reshape(-1, 2)
    return "".join(f"{a:e}{sep}{b:e}{end}" for a, b in v)


class ParticleDump:
    """Asynchronous dump_particles (src/helpers.h:31-61).  enqueue() computes
    the printed values on the device and starts their copy into pinned host
    memory on the stream; write() waits for that copy only and appends the
    reference's line ("%e  %e " per particle, then a newline) to a file.  A
    time loop enqueues at step k and writes before enqueueing at k + 1, so the
    copy overlaps the next step's kernels."""

    def __init__(self, particles: ParticleList):
        R = torch.float32 if particles.precision == capi.CPIC_FLOAT else torch.float64
        n = max(particles.n, 1)
        self._dev = torch.empty(2 * n, dtype=R, device=particles.buf.device)
        self._host = torch.empty(2 * n, dtype=R).pin_memory()
        self._event = torch.cuda.Event()
        self._pending = False
        self._n = particles.n

    def enqueue(self, particles: ParticleList, xmin, dx, nx, ny, nz, ng, boundary=Boundary.Periodic,
                *, stream=None) -> None:
        capi.load().call("cpic_particle_dump_values", particles.ptr, particles.n, particles.vl,
                         C.byref(_grid(nx, ny, nz, ng, boundary)), particles.precision, float(xmin),
                         float(dx), self._dev.data_ptr(), _stream(stream))
        s = torch.cuda.current_stream() if stream is None else stream
        with torch.cuda.stream(s):
            self._host.copy_(self._dev, non_blocking=True)
            self._event.record(s)
        self._pending = True

    def write(self, fp) -> None:
        if not self._pending:
            return
        self._event.synchronize()
        fp.write(_fmt_pairs(self._host[: 2 * self._n].numpy(), "  ", " ") + "\n")
        self._pending = False


def dump_particles(fp, particles: ParticleList, xmin, ymin, zmin, dx, dy, dz, nx, ny, nz, ng) -> None:
    """dump_particles (src/helpers.h:31-61), synchronous: one line with the
    x position and ux of every particle."""
    d = ParticleDump(particles)
    d.enqueue(particles, xmin, dx, nx, ny, nz, ng)
    d.write(fp)


class FieldDump:
    """Asynchronous Field_Solver::dump_fields (src/fields.h:318-350): x and ex
    along the first x row, "%e %e" lines then a blank line."""

    def __init__(self, fields: FieldArray, nx: int):
        R = torch.float32 if fields.precision == capi.CPIC_FLOAT else torch.float64
        self._dev = torch.empty(2 * max(nx, 1), dtype=R, device=fields.buf.device)
        self._host = torch.empty(2 * max(nx, 1), dtype=R).pin_memory()
        self._event = torch.cuda.Event()
        self._pending = False
        self._nx = nx

    def enqueue(self, fields: FieldArray, xmin, dx, nx, ny, nz, ng, boundary=Boundary.Periodic,
                *, stream=None) -> None:
        capi.load().call("cpic_field_dump_values", fields.ptr, C.byref(_grid(nx, ny, nz, ng, boundary)),
                         fields.precision, float(xmin), float(dx), self._dev.data_ptr(), _stream(stream))
        s = torch.cuda.current_stream() if stream is None else stream
        with torch.cuda.stream(s):
            self._host.copy_(self._dev, non_blocking=True)
            self._event.record(s)
        self._pending = True

    def write(self, fp) -> None:
        if not self._pending:
            return
        self._event.synchronize()
        fp.write(_fmt_pairs(self._host[: 2 * self._nx].numpy(), " ", "\n") + "\n\n")
        self._pending = False


# ---------------------------------------------------------------- sort
class Sorter:
    """Counting sort of a particle list by cell (scratch owned by this object).

    double_buffer=True keeps a second particle buffer instead of the in-place
    sort's copy: each sort gathers into it and the list swaps buffers (same
    memory, one 2 x list-size copy less per sort).  The list's buffer object
    changes; hold the ParticleList, not its buffer.

    steps_ahead > 0 (double-buffered only) keys each particle by the cell it
    reaches that many free-streaming pushes ahead (cpic_sort_particles_ahead_into);
    `ahead` = (grid dims (nx, ny, nz), (cdt_dx, cdt_dy, cdt_dz)) is then required."""

    def __init__(self, particles: ParticleList, num_cells: int, double_buffer: bool = False,
                 steps_ahead: int = 0, ahead=None):
        lib = capi.load()
        self.num_cells = int(num_cells)
        self.double_buffer = bool(double_buffer)
        self.steps_ahead = int(steps_ahead)
        if self.steps_ahead < 0:
            raise ValueError("steps_ahead must be >= 0")
        if self.steps_ahead:
            if not self.double_buffer or ahead is None:
                raise ValueError("look-ahead keys need double_buffer=True and the grid and cdt's")
            (nx, ny, nz), cdt = ahead
            self._grid = capi.make_grid(nx, ny, nz)
            self._prm = capi.CpicPushParams(0.0, *[float(v) for v in cdt], 0.0, particles.precision,
                                            particles.vl, 0, 0)
        fn = "cpic_sort_into_scratch_bytes" if self.double_buffer else "cpic_sort_scratch_bytes"
        nbytes = lib.raw(fn)(particles.n, self.num_cells, particles.precision, particles.vl)
        if nbytes == 0:
            raise capi.CpicError(fn, capi.CPIC_EINVAL, "bad arguments")
        self.scratch = torch.empty(nbytes, dtype=torch.uint8, device=particles.buf.device)
        self.spare = torch.empty_like(particles.buf) if self.double_buffer else None

    def __call__(self, particles: ParticleList, *, stream=None) -> None:
        lib = capi.load()
        if self.steps_ahead:
            lib.call("cpic_sort_particles_ahead_into", particles.ptr, self.spare.data_ptr(), particles.n,
                     C.byref(self._grid), C.byref(self._prm), self.steps_ahead, self.scratch.data_ptr(),
                     self.scratch.numel(), _stream(stream))
            particles.buf, self.spare = self.spare, particles.buf
            return
        if self.double_buffer:
            lib.call("cpic_sort_particles_into", particles.ptr, self.spare.data_ptr(), particles.n,
                     self.num_cells, particles.precision, particles.vl, self.scratch.data_ptr(),
                     self.scratch.numel(), _stream(stream))
            particles.buf, self.spare = self.spare, particles.buf
            return
        lib.call("cpic_sort_particles", particles.ptr, particles.n, self.num_cells,
                 particles.precision, particles.vl, self.scratch.data_ptr(), self.scratch.numel(),
                 _stream(stream))


def sort_particles(particles: ParticleList, num_cells: int, *, stream=None) -> None:
    Sorter(particles, num_cells)(particles, stream=stream)


# ---------------------------------------------------------------- diagnostics
class Diagnostics:
    """FP64 charge density, Gauss residual (div E - rho/eps0) and kinetic
    energy on the device (no counterpart in the reference)."""

    def __init__(self, num_cells: int, device=None):
        lib = capi.load()
        dev = torch.device(device if device is not None else "cuda")
        self.rho = torch.zeros(num_cells, dtype=torch.float64, device=dev)
        self.scratch = torch.zeros(lib.raw("cpic_diag_scratch_bytes")(), dtype=torch.uint8, device=dev)
        self.out = torch.zeros(4, dtype=torch.float64, device=dev)

    def charge_density(self, particles: ParticleList, nx, ny, nz, ng, qsp, dx, dy, dz, *,
                       boundary=Boundary.Periodic, stream=None) -> torch.Tensor:
        capi.load().call("cpic_charge_density", particles.ptr, particles.n,
                         C.byref(_grid(nx, ny, nz, ng, boundary)), particles.precision, particles.vl,
                         float(qsp), float(dx), float(dy), float(dz), self.rho.data_ptr(),
                         _STATUS.get().data_ptr(), _stream(stream))
        return self.rho

    def gauss_residual(self, fields: FieldArray, rho: torch.Tensor, nx, ny, nz, ng, dx, dy, dz,
                       eps0=1.0, ref: torch.Tensor = None, resid: torch.Tensor = None, *,
                       boundary=Boundary.Periodic, stream=None) -> torch.Tensor:
        """Returns a device tensor {max|r|, sum r^2, sum (rho/eps0)^2}."""
        out = torch.zeros(3, dtype=torch.float64, device=fields.buf.device)
        capi.load().call("cpic_gauss_residual", fields.ptr, rho.data_ptr(),
                         ref.data_ptr() if ref is not None else None, float(eps0), float(dx),
                         float(dy), float(dz), C.byref(_grid(nx, ny, nz, ng, boundary)),
                         fields.precision, resid.data_ptr() if resid is not None else None,
                         out.data_ptr(), self.scratch.data_ptr(), self.scratch.numel(), _stream(stream))
        return out

    def kinetic_energy(self, particles: ParticleList, mc2=1.0, *, stream=None) -> torch.Tensor:
        out = torch.zeros(1, dtype=torch.float64, device=particles.buf.device)
        capi.load().call("cpic_kinetic_energy", particles.ptr, particles.n, particles.precision,
                         particles.vl, float(mc2), out.data_ptr(), self.scratch.data_ptr(),
                         self.scratch.numel(), _stream(stream))
        return out
