"""Device containers with the reference's layouts.

Stand-ins for the reference's Cabana/Kokkos containers (src/types.h):
ParticleList ~ particle_list_t, InterpolatorArray ~ interpolator_array_t,
AccumulatorArray ~ accumulator_array_t, FieldArray ~ field_array_t.  Device
memory comes from torch (the plumbing); the kernels see raw pointers through
the C ABI.  Layout conversion to and from host arrays is in layout.py.
"""
from __future__ import annotations

import numpy as np
import torch

from . import layout as L


def _dev(device):
    return torch.device(device if device is not None else "cuda")


def _torch_real(real: np.dtype):
    return torch.float32 if np.dtype(real) == np.float32 else torch.float64


_COPY_STREAMS = {}


def copy_streams(dev, pieces: int) -> list:
    """`pieces` side streams for host <-> device copies (created once)."""
    streams = _COPY_STREAMS.get(dev)
    if streams is None or len(streams) < pieces:
        streams = [torch.cuda.Stream(dev) for _ in range(pieces)]
        _COPY_STREAMS[dev] = streams
    return streams


def block_pieces(n: int, vl: int, pieces: int) -> list:
    """Splits n particles into at most `pieces` runs of whole AoSoA blocks:
    [(start, count)]."""
    blocks = -(-n // vl)
    per = -(-blocks // max(1, pieces))
    out = []
    for b0 in range(0, blocks, per):
        start = b0 * vl
        out.append((start, min(n, (b0 + per) * vl) - start))
    return out


def copy_in_pieces(dst: torch.Tensor, src: torch.Tensor, pieces: int = 8) -> None:
    """dst.copy_(src) between pinned host and device memory as `pieces`
    asynchronous copies on side streams, so that several copy engines move
    the bytes at once.  Ordered after the current stream's earlier work; the
    current stream waits for all pieces.  One cudaMemcpyAsync per piece."""
    assert dst.numel() == src.numel() and dst.dtype == src.dtype
    dev = dst.device if dst.is_cuda else src.device
    cur = torch.cuda.current_stream(dev)
    streams = copy_streams(dev, pieces)
    n = dst.numel()
    step = -(-n // pieces)
    start = torch.cuda.Event()
    start.record(cur)
    dev_t = dst if dst.is_cuda else src
    for i in range(pieces):
        a, b = i * step, min(n, (i + 1) * step)
        if a >= b:
            break
        s = streams[i]
        s.wait_event(start)
        with torch.cuda.stream(s):
            dst[a:b].copy_(src[a:b], non_blocking=True)
        dev_t.record_stream(s)
        done = torch.cuda.Event()
        done.record(s)
        cur.wait_event(done)


class ParticleList:
    """particle_list_t: Cabana AoSoA<real_t x7, int> of n particles."""

    def __init__(self, n: int, real=np.float32, vl: int = 32, device=None):
        self.n = int(n)
        self.real = np.dtype(real)
        self.vl = int(vl)
        self.nbytes = L.particle_list_bytes(self.n, self.real, self.vl)
        self.buf = torch.zeros(max(self.nbytes, 16), dtype=torch.uint8, device=_dev(device))

    @property
    def precision(self) -> int:
        return self.real.itemsize

    @property
    def ptr(self) -> int:
        return self.buf.data_ptr()

    def size(self) -> int:
        return self.n

    def upload(self, host) -> "ParticleList":
        """host: dict of member arrays or packed AoSoA bytes."""
        packed = host if isinstance(host, np.ndarray) else L.pack_particles(host, self.real, self.vl)
        assert packed.nbytes == self.nbytes, (packed.nbytes, self.nbytes)
        self.buf[: self.nbytes].copy_(torch.from_numpy(packed.view(np.uint8)))
        return self

    def upload_pinned(self, pinned: torch.Tensor, pieces: int = 8) -> "ParticleList":
        """Asynchronous upload of packed AoSoA bytes from a pinned host tensor
        (uint8, nbytes), split over several copy engines; stream-ordered."""
        copy_in_pieces(self.buf[: self.nbytes], pinned, pieces)
        return self

    def download_pinned(self, pinned: torch.Tensor, pieces: int = 8) -> torch.Tensor:
        """Asynchronous download of the AoSoA bytes into a pinned host tensor;
        complete once the current stream has reached this point."""
        copy_in_pieces(pinned, self.buf[: self.nbytes], pieces)
        return pinned

    def view(self, start: int, count: int) -> "ParticleList":
        """Particles [start, start + count) as a particle list sharing this
        list's memory (start a multiple of the vector length, so the view is
        whole AoSoA blocks)."""
        if start % self.vl or start < 0 or count < 0 or start + count > self.n:
            raise ValueError("a view starts on an AoSoA block and lies inside the list")
        v = ParticleList.__new__(ParticleList)
        v.n, v.real, v.vl = int(count), self.real, self.vl
        v.nbytes = L.particle_list_bytes(v.n, self.real, self.vl)
        off = (start // self.vl) * L.particle_block_bytes(self.real, self.vl)
        v.buf = self.buf[off: off + max(v.nbytes, 16)]
        return v

    def download_bytes(self) -> np.ndarray:
        return self.buf[: self.nbytes].cpu().numpy()

    def download(self) -> dict:
        return L.unpack_particles(self.download_bytes(), self.n, self.real, self.vl)


class _CellArray:
    members = 0

    def __init__(self, num_cells: int, real=np.float32, device=None):
        self.num_cells = int(num_cells)
        self.real = np.dtype(real)
        n = L.cell_array_bytes(self.num_cells, self.members, self.real) // self.real.itemsize
        self.buf = torch.zeros(n, dtype=_torch_real(self.real), device=_dev(device))

    @property
    def precision(self) -> int:
        return self.real.itemsize

    @property
    def ptr(self) -> int:
        return self.buf.data_ptr()

    def size(self) -> int:
        return self.num_cells

    def set_members(self, vals: np.ndarray) -> None:
        """vals: (num_cells, members) host array."""
        self.buf.copy_(torch.from_numpy(L.pack_cells(np.asarray(vals), self.real)))

    def get_members(self) -> np.ndarray:
        return L.unpack_cells(self.buf.cpu().numpy(), self.num_cells, self.members)


class InterpolatorArray(_CellArray):
    """interpolator_array_t: AoSoA of 18 coefficients per cell, 32-cell blocks."""
    members = L.INTERP_MEMBERS


class FieldArray(_CellArray):
    """field_array_t: AoSoA of ex ey ez cbx cby cbz jfx jfy jfz, 32-cell blocks."""
    members = L.FIELD_MEMBERS


class AccumulatorArray:
    """accumulator_array_t: View<real_t*[3][4]> in LayoutRight ([cell][comp][q],
    the reference's host build), or with layout="left" in Kokkos' LayoutLeft
    (the Kokkos-Cuda default: value (comp, q) of cell c at c + num_cells (comp
    + 3 q), stored here as a [q][comp][cell] tensor).  get() and set() take
    (num_cells, 3, 4) values in either layout."""

    def __init__(self, num_cells: int, real=np.float32, device=None, layout: str = "right"):
        if layout not in ("right", "left"):
            raise ValueError("layout is 'right' or 'left'")
        self.num_cells = int(num_cells)
        self.real = np.dtype(real)
        self.layout = layout
        shape = (self.num_cells, 3, 4) if layout == "right" else (4, 3, self.num_cells)
        self.buf = torch.zeros(shape, dtype=_torch_real(self.real), device=_dev(device))

    @property
    def precision(self) -> int:
        return self.real.itemsize

    @property
    def ptr(self) -> int:
        return self.buf.data_ptr()

    def size(self) -> int:
        return self.num_cells

    def get(self) -> np.ndarray:
        a = self.buf.cpu().numpy()
        return a if self.layout == "right" else np.ascontiguousarray(a.transpose(2, 1, 0))

    def set(self, vals: np.ndarray) -> None:
        v = np.asarray(vals, self.real).reshape(self.num_cells, 3, 4)
        if self.layout == "left":
            v = np.ascontiguousarray(v.transpose(2, 1, 0))
        self.buf.copy_(torch.from_numpy(v))
