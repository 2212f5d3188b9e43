"""Input decks: run parameters and particle initializers.

Deck mirrors the reference's _Input_Deck (src/input/deck.h:161-348) and the
constants main() derives from it (example/example.cpp:77-113,179-181), computed
in real_t with the reference's C++ promotion rules (a double literal promotes
the expression to double; the result is rounded to real_t on assignment), so
a float deck here gives the same bits as the reference's float build.

Initializers:
  default_particles  the reference's default Particle_Initializer
                     (src/input/deck.h:79-158), used by its 2stream-em test deck
  two_stream_1d      seeded two-beam plasma along x with a sin(kx) perturbation
  thermal            seeded uniform Maxwellian plasma, particles in cell order
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np

from . import layout as L

f64 = np.float64


@dataclass
class Deck:
    nx: int = 16
    ny: int = 1
    nz: int = 1
    num_ghosts: int = 1
    nppc: int = 1
    num_steps: int = 2
    dt: float = 1.0
    c: float = 1.0
    eps: float = 1.0
    me: float = 1.0
    ec: float = 1.0
    n0: float = 1.0
    v0: float = 1.0
    len_x_global: float = 1.0
    len_y_global: float = 1.0
    len_z_global: float = 1.0
    boundary: int = 1           # Periodic
    precision: int = 4          # sizeof(real_t)
    vl: int = 32                # particle AoSoA vector length
    name: str = "deck"
    extra: dict = field(default_factory=dict)

    @property
    def R(self):
        return np.float32 if self.precision == 4 else np.float64

    @property
    def num_cells(self) -> int:
        g = 2 * self.num_ghosts
        return (self.nx + g) * (self.ny + g) * (self.nz + g)

    @property
    def num_interior(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def num_particles(self) -> int:
        return self.nx * self.ny * self.nz * self.nppc

    def derived(self) -> dict:
        """derive_params() (deck.h:323-348) and main()'s constants (example.cpp:77-181)."""
        R = self.R
        c, eps, me, n0 = R(self.c), R(self.eps), R(self.me), R(self.n0)
        qsp = R(-R(self.ec))
        dt = R(self.dt)
        lx, ly, lz = R(self.len_x_global), R(self.len_y_global), R(self.len_z_global)
        dx, dy, dz = R(lx / R(self.nx)), R(ly / R(self.ny)), R(lz / R(self.nz))
        Ne = R(self.num_particles)
        Npe = R(R(R(n0 * lx) * ly) * lz)
        frac = R(1.0)
        d = dict(
            dx=dx, dy=dy, dz=dz, dt=dt, c=c, eps=eps, me=me, qsp=qsp, n0=n0,
            len_x=lx, len_y=ly, len_z=lz, Ne=Ne, Npe=Npe,
            dxp=R(np.float32(2.0) / np.float32(self.nppc)),
            qdt_2mc=R(R(qsp * dt) / R(R(R(2) * me) * c)),
            cdt_dx=R(R(c * dt) / dx), cdt_dy=R(R(c * dt) / dy), cdt_dz=R(R(c * dt) / dz),
            dt_eps0=R(dt / eps),
            we=R(Npe / Ne),
            px=R(R(R(frac * c) * dt) / dx) if self.nx > 1 else R(0),
            py=R(R(R(frac * c) * dt) / dy) if self.ny > 1 else R(0),
            pz=R(R(R(frac * c) * dt) / dz) if self.nz > 1 else R(0),
            num_cells=self.num_cells, num_particles=self.num_particles,
        )
        return d


def courant_length(lx, ly, lz, nx, ny, nz, R=np.float32):
    """_Input_Deck::courant_length (deck.h:191-198), in real_t."""
    lx, ly, lz = R(lx), R(ly), R(lz)
    w1 = R(0)
    if nx > 1:
        w0 = R(R(nx) / lx); w1 = R(w1 + R(w0 * w0))
    if ny > 1:
        w0 = R(R(ny) / ly); w1 = R(w1 + R(w0 * w0))
    if nz > 1:
        w0 = R(R(nz) / lz); w1 = R(w1 + R(w0 * w0))
    return R(math.sqrt(f64(R(R(1) / w1))))


# ---------------------------------------------------------------- decks
def two_stream_em(precision: int = 4, vl: int = 32, num_steps: int = 6000) -> Deck:
    """The 2stream-em deck of the reference's regression test
    (tests/energy_comparison/2stream-em.cxx:81-114; same as deck.h:432-464)."""
    R = np.float32 if precision == 4 else np.float64
    v0 = R(0.0866025403784439)
    gam = R(1.0 / math.sqrt(1.0 - f64(R(v0 * v0))))
    len_y = R(0.628318530717959 * (f64(gam) * math.sqrt(f64(gam))))
    d = Deck(nx=1, ny=32, nz=1, nppc=100, num_steps=num_steps, v0=float(v0),
             len_x_global=1.0, len_y_global=float(len_y), len_z_global=1.0, n0=2.0,
             precision=precision, vl=vl, name="2stream-em")
    cl = courant_length(1.0, len_y, 1.0, 1, 32, 1, R)
    d.dt = float(R(0.99 * f64(cl) / f64(R(d.c))))
    return d


def two_stream_1d(precision: int = 4, vl: int = 32, num_steps: int = 2000, nx: int = 32,
                  ppc_per_beam: int = 32, drift: float = 0.2, amp: float = 1e-3, mode: int = 3,
                  seed: int = 1) -> Deck:
    """Two cold electron beams u_x = +-drift along x in a periodic nx x 1 x 1 box of
    length 2*pi/mode, dt = 0.98 Courant, n0 = 1 (wpe = 1), velocity perturbation
    amp*drift*sin(mode*x)."""
    R = np.float32 if precision == 4 else np.float64
    lx = 2.0 * math.pi / 3.0
    d = Deck(nx=nx, ny=1, nz=1, nppc=2 * ppc_per_beam, num_steps=num_steps, v0=drift,
             len_x_global=lx, n0=1.0, precision=precision, vl=vl, name="two-stream-1d",
             extra=dict(amp=amp, mode=mode, seed=seed))
    d.dt = float(R(0.98 * f64(courant_length(lx, 1.0, 1.0, nx, 1, 1, R))))
    return d


def thermal(n: int = 128, ppc: int = 64, precision: int = 4, vl: int = 32, uth: float = 0.05,
            dx: float = 0.05, courant: float = 0.7, num_steps: int = 100, seed: int = 2024) -> Deck:
    """Uniform thermal plasma: n^3 periodic cells of size dx (one Debye length
    u_th/w_pe for dx = u_th), ppc electrons per cell with uniform offsets in
    [-1,1] and Maxwellian momenta u_th per component, zero initial fields,
    n0 = 1 (w_pe = 1), dt = courant x the Courant limit."""
    R = np.float32 if precision == 4 else np.float64
    L_ = n * dx
    d = Deck(nx=n, ny=n, nz=n, nppc=ppc, num_steps=num_steps, v0=0.0,
             len_x_global=L_, len_y_global=L_, len_z_global=L_, n0=1.0,
             precision=precision, vl=vl, name=f"thermal-{n}^3-{ppc}ppc",
             extra=dict(uth=uth, seed=seed))
    d.dt = float(R(courant * f64(courant_length(L_, L_, L_, n, n, n, R))))
    return d


# ---------------------------------------------------------------- initializers
def default_particles(deck: Deck) -> dict:
    """Default Particle_Initializer::init (deck.h:79-158): pairs of +/- beams
    along x, stratified in y, 1e-4 sin perturbation.  Float arithmetic as the
    reference's float or double build."""
    R = deck.R
    p = deck.derived()
    n = deck.num_particles
    nx, ny, nppc = deck.nx, deck.ny, deck.nppc
    dxp, w, v0 = p["dxp"], p["we"], R(deck.v0)
    pi2 = np.arange(n, dtype=np.int64)
    sign = np.where(pi2 % 2 == 0, 1, -1)
    pi = pi2 // 2
    pic = (2 * pi) % nppc
    x = (((pic.astype(R) * dxp).astype(f64) + 0.5 * f64(dxp)) - 1.0).astype(R)
    pre_ghost = (2 * pi) // nppc
    cell = pre_ghost * (nx + 2) + (nx + 2) * (ny + 2) + (nx + 2) + 1
    gam = R(1.0 / math.sqrt(1.0 - f64(R(v0 * v0))))
    na = (0.0001 * np.sin(2.0 * 3.1415926 * ((x.astype(f64) + 1.0 + pre_ghost * 2) / (2 * ny)))).astype(R)
    sv = (sign.astype(R) * v0) * gam
    ux = (sv.astype(f64) * (1.0 + (na * sign.astype(R)).astype(f64))).astype(R)
    z = np.zeros(n, R)
    return dict(x=z.copy(), y=x, z=z.copy(), ux=ux, uy=z.copy(), uz=z.copy(),
                w=np.full(n, w, R), cell=cell.astype(np.int32))


def two_stream_1d_particles(deck: Deck) -> dict:
    R = deck.R
    p = deck.derived()
    rng = np.random.default_rng(deck.extra.get("seed", 1))
    n = deck.num_particles
    nx = deck.nx
    amp, mode, drift = deck.extra.get("amp", 1e-3), deck.extra.get("mode", 3), deck.v0
    # global x in [0, Lx): cell = floor(x/dx), offset in [-1, 1)
    X = rng.random(n) * deck.len_x_global
    ix = np.minimum((X / deck.len_x_global * nx).astype(np.int64), nx - 1)
    off = (X / deck.len_x_global * nx - ix) * 2.0 - 1.0
    sign = np.where(np.arange(n) % 2 == 0, 1.0, -1.0)
    ux = sign * drift + amp * drift * np.sin(mode * X)
    cell = L.voxel(ix + 1, 1, 1, nx, 1)
    out = dict(x=off.astype(R), y=(rng.random(n) * 2 - 1).astype(R), z=(rng.random(n) * 2 - 1).astype(R),
               ux=ux.astype(R), uy=np.zeros(n, R), uz=np.zeros(n, R),
               w=np.full(n, p["we"], R), cell=cell.astype(np.int32),
               X=X, sign=sign)  # X, sign: the initial-condition parameters' inputs (not packed)
    order = np.argsort(out["cell"], kind="stable")
    return {k: v[order] for k, v in out.items()}


def thermal_particles(deck: Deck, packed: bool = False, n_sample: int = None):
    """Seeded uniform Maxwellian plasma in cell order (ppc particles per
    interior cell, cells in VOXEL order).  With packed=True returns the AoSoA
    bytes directly (avoids a second copy at large sizes).  n_sample limits the
    number of particles generated (every cell keeps its ppc slot pattern: the
    first n_sample particles)."""
    R = deck.R
    p = deck.derived()
    n = deck.num_particles if n_sample is None else int(n_sample)
    rng = np.random.default_rng(deck.extra.get("seed", 2024))
    uth = deck.extra.get("uth", 0.05)
    nx, ny = deck.nx, deck.ny
    k = np.arange(n, dtype=np.int64) // deck.nppc
    ix = k % nx
    iy = (k // nx) % ny
    iz = k // (nx * ny)
    cell = L.voxel(ix + 1, iy + 1, iz + 1, nx, ny).astype(np.int32)
    del k, ix, iy, iz
    dt = np.float32 if R is np.float32 else np.float64
    out = dict(
        x=(rng.random(n, dtype=dt) * 2 - 1).astype(R, copy=False),
        y=(rng.random(n, dtype=dt) * 2 - 1).astype(R, copy=False),
        z=(rng.random(n, dtype=dt) * 2 - 1).astype(R, copy=False),
        ux=(rng.standard_normal(n, dtype=dt) * uth).astype(R, copy=False),
        uy=(rng.standard_normal(n, dtype=dt) * uth).astype(R, copy=False),
        uz=(rng.standard_normal(n, dtype=dt) * uth).astype(R, copy=False),
        w=np.full(n, p["we"], R),
        cell=cell,
    )
    if packed:
        return L.pack_particles(out, R, deck.vl)
    return out


def initial_particles(deck: Deck) -> dict:
    if deck.name == "2stream-em":
        return default_particles(deck)
    if deck.name == "two-stream-1d":
        return two_stream_1d_particles(deck)
    return thermal_particles(deck)
