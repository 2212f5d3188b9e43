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
  diocotron          3-D electron column (annulus) in a uniform axial B, loaded
                     at the local E x B drift of its own field, which is solved
                     on the grid at t = 0 (discrete Poisson equation, FFT)
  diocotron_slab     the reference's decks/dioctron_3d.cxx: a y-strip of cold
                     electrons in a uniform B_z with a sheared E_y field
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
    n_particles: int = 0        # particle count when not nppc per interior cell

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
        if self.n_particles > 0:
            return self.n_particles
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


_PHILOX_M = (np.uint64(0xD2511F53), np.uint64(0xCD9E8D57))
_PHILOX_W = (0x9E3779B9, 0xBB67AE85)
_U32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0: int, k1: int):
    """Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) over arrays of
    counters: per round two 32x32->64 products of counter words 0 and 2,
    their high halves mixed with words 1 and 3 and the key, the key bumped by
    the Weyl constants.  Returns the four output words (uint32 arrays).  The
    same generator as the device loader (csrc/init.cu)."""
    shape = np.broadcast(c0, c1, c2, c3).shape
    c0, c1, c2, c3 = (np.broadcast_to(np.asarray(c, np.uint64), shape).astype(np.uint64) for c in (c0, c1, c2, c3))
    k0, k1 = int(k0) & 0xFFFFFFFF, int(k1) & 0xFFFFFFFF
    for _ in range(10):
        p0 = c0 * _PHILOX_M[0]
        p1 = c2 * _PHILOX_M[1]
        c0, c1, c2, c3 = ((p1 >> np.uint64(32)) ^ c1 ^ np.uint64(k0), p1 & _U32,
                          (p0 >> np.uint64(32)) ^ c3 ^ np.uint64(k1), p0 & _U32)
        k0 = (k0 + _PHILOX_W[0]) & 0xFFFFFFFF
        k1 = (k1 + _PHILOX_W[1]) & 0xFFFFFFFF
    return tuple(c.astype(np.uint32) for c in (c0, c1, c2, c3))


def _thermal_values(p: np.ndarray, R, uth: float, seed: int):
    """x, y, z, ux, uy, uz of particles p (uint64 indices): counters (p, 0) and
    (p, 1) under key `seed`; offsets 2u - 1 from 24 (FP32) or 32 (FP64) bits,
    Box-Muller normals in double rounded once to real_t."""
    lo, hi = p & _U32, p >> np.uint64(32)
    k0, k1 = seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF
    a = philox4x32_10(lo, hi, 0, 0, k0, k1)
    b = philox4x32_10(lo, hi, 1, 0, k0, k1)
    if np.dtype(R) == np.float32:
        off = [(a[i] >> np.uint32(8)).astype(np.float32) * np.float32(2.0 ** -23) - np.float32(1) for i in range(3)]
    else:
        off = [a[i].astype(np.float64) * 2.0 ** -31 - 1.0 for i in range(3)]
    r1 = np.sqrt(-2.0 * np.log((a[3].astype(np.float64) + 1.0) * 2.0 ** -32))
    r2 = np.sqrt(-2.0 * np.log((b[1].astype(np.float64) + 1.0) * 2.0 ** -32))
    t1 = np.pi * (2.0 * (b[0].astype(np.float64) * 2.0 ** -32))
    t2 = np.pi * (2.0 * (b[2].astype(np.float64) * 2.0 ** -32))
    mom = [(uth * (r1 * np.cos(t1))).astype(R), (uth * (r1 * np.sin(t1))).astype(R),
           (uth * (r2 * np.cos(t2))).astype(R)]
    return off + mom


def thermal_particles(deck: Deck, packed: bool = False, n_sample: int = None):
    """Seeded uniform Maxwellian plasma in cell order (ppc particles per
    interior cell, cells in VOXEL order), on the host: the numpy restatement
    of the device loader (thermal_particles_device, csrc/init.cu), particle p
    drawing from Philox4x32-10 counters (p, 0) and (p, 1) under the deck's
    seed.  Offsets and cells are bit-identical to the device's; momenta agree
    to the rounding of the libm and CUDA log/cos.  With packed=True returns the
    AoSoA bytes.  n_sample limits the number of particles generated (the
    first n_sample of the deck's sequence)."""
    R = deck.R
    p = deck.derived()
    n = deck.num_particles if n_sample is None else int(n_sample)
    seed = int(deck.extra.get("seed", 2024))
    uth = float(deck.extra.get("uth", 0.05))
    nx, ny = deck.nx, deck.ny
    out = {k: np.empty(n, R) for k in L.PARTICLE_REAL_MEMBERS}
    out["cell"] = np.empty(n, np.int32)
    out["w"][:] = p["we"]
    chunk = 1 << 22
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        idx = np.arange(a, b, dtype=np.uint64)
        k = (idx // np.uint64(deck.nppc)).astype(np.int64)
        out["cell"][a:b] = L.voxel(k % nx + 1, (k // nx) % ny + 1, k // (nx * ny) + 1, nx, ny)
        for key, v in zip(("x", "y", "z", "ux", "uy", "uz"), _thermal_values(idx, R, uth, seed)):
            out[key][a:b] = v
    if packed:
        return L.pack_particles(out, R, deck.vl)
    return out


def is_thermal(deck: Deck) -> bool:
    return deck.name.startswith("thermal-")


def thermal_particles_device(deck: Deck, particles=None, device=None, *, stream=None):
    """The thermal plasma generated on the device (cpic_thermal_particles):
    the same particles as thermal_particles, without the host round trip.
    Fills `particles` (a ParticleList of deck.num_particles) or a new one."""
    from . import pic
    from .arrays import ParticleList
    if particles is None:
        particles = ParticleList(deck.num_particles, deck.R, deck.vl, device)
    pic.thermal_particles(particles, deck.nppc, deck.nx, deck.ny, deck.nz,
                          float(deck.extra.get("uth", 0.05)), float(deck.derived()["we"]),
                          int(deck.extra.get("seed", 2024)), stream=stream)
    return particles


# ---------------------------------------------------------------- diocotron
def diocotron(precision: int = 4, vl: int = 32, n=(96, 96, 64), ppc: int = 128, dx: float = 0.2,
              b0: float = 5.0, r_in: float = 0.20, r_out: float = 0.35, amp: float = 0.01,
              mode: int = 3, num_steps: int = 2000, seed: int = 7) -> Deck:
    """3-D diocotron column on an n = (nx, ny, nz) periodic grid of cubic cells
    of size dx (c / w_pe units, c = eps0 = m_e = |q| = 1): uniform axial field
    cB_z = b0 (w_ce / w_pe = b0 at the column's density 1), electrons only in
    the annulus r_in < r / R < r_out around the box axis (R = half the
    transverse width) at ppc particles per cell of annulus volume, an azimuthal
    density perturbation 1 + amp cos(mode theta) carried by the weights, cold
    momenta at the local E x B drift, a uniform neutralising background,
    dt = 0.99 x the Courant limit (as decks/dioctron_3d.cxx)."""
    R = np.float32 if precision == 4 else np.float64
    nx, ny, nz = (int(v) for v in n)
    lx, ly, lz = nx * dx, ny * dx, nz * dx
    rad = 0.5 * min(lx, ly)
    area_cells = math.pi * (r_out ** 2 - r_in ** 2) * rad * rad / (dx * dx)
    npart = int(round(ppc * area_cells * nz))
    npart -= npart % 32 if npart > 64 else 0
    d = Deck(nx=nx, ny=ny, nz=nz, nppc=ppc, num_steps=num_steps, v0=0.0,
             len_x_global=lx, len_y_global=ly, len_z_global=lz, n0=1.0, precision=precision,
             vl=vl, name="diocotron", n_particles=npart,
             extra=dict(b0=b0, r_in=r_in, r_out=r_out, amp=amp, mode=mode, seed=seed, radius=rad))
    d.dt = float(R(0.99 * f64(courant_length(lx, ly, lz, nx, ny, nz, R))))
    return d


def node_charge_density(p: dict, nx: int, ny: int, nz: int, dx: float, dy: float, dz: float,
                        qsp: float) -> np.ndarray:
    """Charge density at the nodes (low corners of the voxels), FP64, as
    (nz, ny, nx) over the interior nodes: trilinear weights of each particle
    to the 8 corners of its voxel, the n + 1 layer folded onto node 1
    (periodic)."""
    sx, sy = nx + 2, ny + 2
    c = p["cell"].astype(np.int64)
    iy, ix = np.divmod(c, sx)
    iz, iy = np.divmod(iy, sy)
    x, y, z = (p[k].astype(np.float64) for k in ("x", "y", "z"))
    q = p["w"].astype(np.float64) * (qsp / (dx * dy * dz))
    rho = np.zeros((nz, ny, nx))
    wx = (0.5 * (1 - x), 0.5 * (1 + x))
    wy = (0.5 * (1 - y), 0.5 * (1 + y))
    wz = (0.5 * (1 - z), 0.5 * (1 + z))
    for a in (0, 1):
        jx = (ix - 1 + a) % nx
        for b in (0, 1):
            jy = (iy - 1 + b) % ny
            for e in (0, 1):
                jz = (iz - 1 + e) % nz
                np.add.at(rho, (jz, jy, jx), q * wx[a] * wy[b] * wz[e])
    return rho


def poisson_edge_fields(rho: np.ndarray, dx: float, dy: float, dz: float, eps0: float = 1.0):
    """E = -grad(phi) on the Yee edges for node charge rho (nz, ny, nx) plus a
    uniform neutralising background: the discrete Poisson equation whose
    divergence is the backward-difference div E at the nodes, solved exactly
    by FFT on the periodic grid.  Returns (ex, ey, ez), each (nz, ny, nx):
    ex[k, j, i] on the edge from node i to node i + 1."""
    nz, ny, nx = rho.shape
    r = rho - rho.mean()
    kx = 2 - 2 * np.cos(2 * np.pi * np.arange(nx) / nx)
    ky = 2 - 2 * np.cos(2 * np.pi * np.arange(ny) / ny)
    kz = 2 - 2 * np.cos(2 * np.pi * np.arange(nz) / nz)
    lap = (kz[:, None, None] / (dz * dz) + ky[None, :, None] / (dy * dy)
           + kx[None, None, :] / (dx * dx))
    lap[0, 0, 0] = 1.0
    ph = np.fft.fftn(r / eps0) / lap
    ph[0, 0, 0] = 0.0
    phi = np.real(np.fft.ifftn(ph))
    ex = -(np.roll(phi, -1, axis=2) - phi) / dx
    ey = -(np.roll(phi, -1, axis=1) - phi) / dy
    ez = -(np.roll(phi, -1, axis=0) - phi) / dz
    return ex, ey, ez


def _edge_fields_to_cells(deck: Deck, ex, ey, ez, cbz: float) -> np.ndarray:
    """(num_cells, 9) field members: E edges of interior voxel (i, j, k) from the
    (nz, ny, nx) arrays, periodic images in the ghost layers, uniform cB_z."""
    nx, ny, nz = deck.nx, deck.ny, deck.nz
    F = np.zeros((nz + 2, ny + 2, nx + 2, 9))
    for m, e in enumerate((ex, ey, ez)):
        F[..., m] = np.pad(e, 1, mode="wrap")
    F[..., 5] = cbz
    return F.reshape(-1, 9).astype(deck.R)


def diocotron_state(deck: Deck, packed: bool = False):
    """(particles, fields) at t = 0 for the diocotron deck; particles in cell
    order, fields as (num_cells, 9) member values."""
    R = deck.R
    ex_ = deck.extra
    rng = np.random.default_rng(ex_.get("seed", 7))
    n = deck.num_particles
    p = deck.derived()
    dx, dy, dz = (float(p[k]) for k in ("dx", "dy", "dz"))
    lx, ly, lz = deck.len_x_global, deck.len_y_global, deck.len_z_global
    rad = ex_["radius"]
    r = np.sqrt(rng.uniform((ex_["r_in"] * rad) ** 2, (ex_["r_out"] * rad) ** 2, n))
    th = rng.uniform(0.0, 2 * np.pi, n)
    X = 0.5 * lx + r * np.cos(th)
    Y = 0.5 * ly + r * np.sin(th)
    Z = rng.uniform(0.0, lz, n)
    gx, gy, gz = X / dx, Y / dy, Z / dz
    ix = np.minimum(np.floor(gx).astype(np.int64), deck.nx - 1)
    iy = np.minimum(np.floor(gy).astype(np.int64), deck.ny - 1)
    iz = np.minimum(np.floor(gz).astype(np.int64), deck.nz - 1)
    ox, oy, oz = 2 * (gx - ix) - 1, 2 * (gy - iy) - 1, 2 * (gz - iz) - 1
    vol = math.pi * (ex_["r_out"] ** 2 - ex_["r_in"] ** 2) * rad * rad * lz
    w = (deck.n0 * vol / n) * (1 + ex_["amp"] * np.cos(ex_["mode"] * th))
    cell = L.voxel(ix + 1, iy + 1, iz + 1, deck.nx, deck.ny).astype(np.int32)
    part = dict(x=ox.astype(R), y=oy.astype(R), z=oz.astype(R), w=w.astype(R), cell=cell)
    # the column's field (and the background's) on the grid, then the drift
    rho = node_charge_density(part, deck.nx, deck.ny, deck.nz, dx, dy, dz, float(p["qsp"]))
    exg, eyg, ezg = poisson_edge_fields(rho, dx, dy, dz, float(p["eps"]))
    fx = 0.5 * (1 - part["x"].astype(f64))
    fy = 0.5 * (1 - part["y"].astype(f64))
    jx, jy, jz = ix, iy, iz
    # edge values bilinear across the voxel (the push's interpolation for z-uniform fields)
    Ex = (fy * exg[jz, jy, jx] + (1 - fy) * exg[jz, (jy + 1) % deck.ny, jx])
    Ey = (fx * eyg[jz, jy, jx] + (1 - fx) * eyg[jz, jy, (jx + 1) % deck.nx])
    b0 = ex_["b0"]
    vx, vy = Ey / b0, -Ex / b0
    gam = 1.0 / np.sqrt(1.0 - np.minimum(vx * vx + vy * vy, 0.99))
    part.update(ux=(gam * vx).astype(R), uy=(gam * vy).astype(R), uz=np.zeros(n, R))
    order = np.argsort(cell, kind="stable")
    part = {k: v[order] for k, v in part.items()}
    fields = _edge_fields_to_cells(deck, exg, eyg, ezg, b0)
    if packed:
        part = L.pack_particles(part, R, deck.vl)
    return part, fields


def diocotron_slab(precision: int = 4, vl: int = 32, num_steps: int = 20000, seed: int = 5) -> Deck:
    """decks/dioctron_3d.cxx: 64 x 64 x 1 cells, Lx = Ly = 16 a (a = 0.1),
    Lz = 1, 5 particles per cell of the box, dt = 0.99 Courant, v0 = 0."""
    R = np.float32 if precision == 4 else np.float64
    a = 0.1
    d = Deck(nx=64, ny=64, nz=1, nppc=5, num_steps=num_steps, v0=0.0, len_x_global=16 * a,
             len_y_global=16 * a, len_z_global=1.0, n0=1.0, precision=precision, vl=vl,
             name="diocotron-slab", extra=dict(a=a, seed=seed))
    d.dt = float(R(R(0.99) * courant_length(d.len_x_global, d.len_y_global, d.len_z_global, 64, 64, 1, R)))
    return d


def diocotron_slab_state(deck: Deck, packed: bool = False):
    """Custom_Particle_Initializer and Custom_Field_Initializer of
    decks/dioctron_3d.cxx:4-165: particles uniform in x over the box and in
    |y| < a, z offset 0 in the first z layer, at rest, weight we; fields
    cB_z = sqrt(20) and E_y = a for y < -a, -a for y > a, -y between, with
    y = ymin + (iy - 0.5) dy.  The reference draws positions with rand(); a
    seeded generator stands in."""
    R = deck.R
    p = deck.derived()
    a = deck.extra["a"]
    rng = np.random.default_rng(deck.extra.get("seed", 5))
    n = deck.num_particles
    nx, ny, nz = deck.nx, deck.ny, deck.nz
    lx, ly = deck.len_x_global, deck.len_y_global
    hx, hy = lx / nx, ly / ny
    xmin, ymin = -0.5 * lx, -0.5 * ly
    gx = (rng.uniform(-0.5 * lx, 0.5 * lx, n) - xmin) / hx
    ix = gx.astype(np.int64)
    ox = 2 * (gx - ix) - 1
    ox = np.where(ix == nx, 1.0, ox); ix = np.where(ix == nx, nx - 1, ix)
    gy = (rng.uniform(-a, a, n) - ymin) / hy
    iy = gy.astype(np.int64)
    oy = 2 * (gy - iy) - 1
    oy = np.where(iy == ny, 1.0, oy); iy = np.where(iy == ny, ny - 1, iy)
    cell = L.voxel(ix + 1, iy + 1, 1, nx, ny).astype(np.int32)
    part = dict(x=ox.astype(R), y=oy.astype(R), z=np.zeros(n, R), ux=np.zeros(n, R),
                uy=np.zeros(n, R), uz=np.zeros(n, R), w=np.full(n, p["we"], R), cell=cell)
    order = np.argsort(cell, kind="stable")
    part = {k: v[order] for k, v in part.items()}
    F = np.zeros((nz + 2, ny + 2, nx + 2, 9))
    jy = np.arange(ny + 2)
    yc = ymin + (jy - 0.5) * float(p["dy"])
    F[..., 1] = np.where(yc < -a, a, np.where(yc > a, -a, -yc))[None, :, None]
    F[..., 5] = math.sqrt(20.0)
    fields = F.reshape(-1, 9).astype(R)
    if packed:
        part = L.pack_particles(part, R, deck.vl)
    return part, fields


def initial_particles(deck: Deck) -> dict:
    if deck.name == "2stream-em":
        return default_particles(deck)
    if deck.name == "two-stream-1d":
        return two_stream_1d_particles(deck)
    if deck.name == "diocotron":
        return diocotron_state(deck)[0]
    if deck.name == "diocotron-slab":
        return diocotron_slab_state(deck)[0]
    return thermal_particles(deck)


def initial_fields(deck: Deck, particles=None):
    """Field members (num_cells, 9) at t = 0 for decks that start with fields,
    else None (all zero, the reference's default Field_Initializer)."""
    if deck.name == "diocotron":
        return diocotron_state(deck)[1]
    if deck.name == "diocotron-slab":
        return diocotron_slab_state(deck)[1]
    return None
