"""Adjoint (reverse-mode) time stepping over the C ABI.  No counterpart in the
reference.

Loss: the field energy after K steps, L = 0.5 sum_interior (E^2 + cB^2) (the
quantity dump_energies prints, src/fields.h:722-763).  The forward run keeps
the particle and field state every `checkpoint` steps; the reverse sweep
recomputes each segment from its checkpoint, storing the per-step states of
that segment only, and runs the transposed step backwards:

  forward step n                         reverse step n
  I  = interp(E, B)                      lambda_(E,B)  -= advance_b^T (B half step 2)
  (P', a) = push(P, I)                   lambda_B += Me^T lambda_E, lambda_J = -cj lambda_E
  J  = unload(a)                         lambda_E -= advance_b^T (B half step 1)
  B  = B - 1/2 Mb E                      lambda_a = unload^T lambda_J
  E  = E - cj J + Me B                   (lambda_P, lambda_I) = push^T(P, I; lambda_P', lambda_a)
  B  = B - 1/2 Mb E                      lambda_(E,B) += interp^T lambda_I

Gradients returned: lambda of the initial particle state (offsets and
momenta, per particle) and of the initial fields.  Cell indices are piecewise
constant.  The torch.autograd.Function wrapper used by the verification
harness lives in tests/, not here.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from . import capi, decks as D, pic
from .arrays import AccumulatorArray, FieldArray, InterpolatorArray, ParticleList
from .simulation import Simulation


class AdjointRun:
    def __init__(self, deck: D.Deck, particles, *, fields_init: np.ndarray = None, checkpoint: int = 20,
                 true_sqrt: bool = False, exact: bool = False, device=None):
        self.deck = deck
        self.p = deck.derived()
        self.C = int(checkpoint)
        self.true_sqrt = bool(true_sqrt)
        self.exact = bool(exact)
        self.sim = Simulation(deck, particles, device=device, max_steps=1, exact=exact)
        self.sim.true_sqrt = self.true_sqrt
        if fields_init is not None:
            self.sim.fields.set_members(fields_init)
        R = deck.R
        nc = deck.num_cells
        dev = self.sim.device
        self.lam_fields = FieldArray(nc, R, dev)
        # the interpolator adjoint in cell-major rows (CPIC_ADJ_INTERP_ROWS): a
        # particle's 18 coefficient adjoints land in one or two lines
        self.lam_interp_rows = torch.zeros(nc * capi.CPIC_ADJ_INTERP_ROW,
                                           dtype=torch.float32 if R == np.float32 else torch.float64, device=dev)
        self.lam_acc = AccumulatorArray(nc, R, dev)
        self.lam_part = ParticleList(deck.num_particles, R, deck.vl, dev)
        self.checkpoints = []
        self.K = 0
        self.timing = {}
        # device memory for the reverse sweep, allocated once: per step of a
        # segment, the particles before the step (the first step's are the
        # checkpoint's) and the step's interpolator array; the checkpoint
        # buffers are kept and reused across runs
        self._seg_P = [torch.empty_like(self.sim.particles.buf) for _ in range(self.C - 1)]
        self._seg_I = [torch.empty_like(self.sim.interpolators.buf) for _ in range(self.C)]
        self._ck_bufs = []

    # ------------------------------------------------------------ forward
    def _save(self, i: int):
        """Copies the particle and field state into checkpoint buffer i."""
        s = self.sim
        while len(self._ck_bufs) <= i:
            self._ck_bufs.append((torch.empty_like(s.particles.buf), torch.empty_like(s.fields.buf)))
        P, F = self._ck_bufs[i]
        P.copy_(s.particles.buf)
        F.copy_(s.fields.buf)
        return (P, F)

    def _restore(self, ck):
        s = self.sim
        s.particles.buf.copy_(ck[0])
        s.fields.buf.copy_(ck[1])

    def _step(self, out: torch.Tensor = None, interp_only: bool = False):
        """One forward step.  out: push out of place into this particle buffer
        (the list keeps the state before the step); interp_only: stop after
        the interpolator load."""
        s = self.sim
        d, p = s.deck, s.p
        nx, ny, nz, ng = d.nx, d.ny, d.nz, d.num_ghosts
        pic.load_interpolator_array(s.fields, s.interpolators, nx, ny, nz, ng)
        if interp_only:
            return
        pic.clear_accumulator_array(s.fields, s.accumulators, nx, ny, nz)
        args = (s.interpolators, p["qdt_2mc"], p["cdt_dx"], p["cdt_dy"], p["cdt_dz"], p["qsp"], s.accumulators,
                None, nx, ny, nz, ng, d.boundary)
        if out is None:
            pic.push(s.particles, *args, true_sqrt=self.true_sqrt, exact=self.exact)
        else:
            pic.push_into(s.particles, out, *args, true_sqrt=self.true_sqrt, exact=self.exact)
        pic.unload_accumulator_array(s.fields, s.accumulators, nx, ny, nz, ng, p["dx"], p["dy"], p["dz"], p["dt"])
        h = d.R(0.5)
        s.solver.advance_b(s.fields, d.R(h * p["px"]), d.R(h * p["py"]), d.R(h * p["pz"]), nx, ny, nz, ng)
        s.solver.advance_e(s.fields, p["px"], p["py"], p["pz"], nx, ny, nz, ng, p["dt_eps0"])
        s.solver.advance_b(s.fields, d.R(h * p["px"]), d.R(h * p["py"]), d.R(h * p["pz"]), nx, ny, nz, ng)

    def reset(self) -> None:
        """Back to the initial state (checkpoint 0 of the last forward run)."""
        if self.checkpoints:
            self._restore(self.checkpoints[0])

    def forward(self, K: int) -> float:
        """Runs K steps from the initial state; returns the loss (double)."""
        self.K = int(K)
        self.checkpoints = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for n in range(self.K):
            if n % self.C == 0:
                self.checkpoints.append(self._save(len(self.checkpoints)))
            self._step()
        torch.cuda.synchronize()
        self.timing["forward_s"] = time.perf_counter() - t0
        d = self.deck
        e = self.sim.solver.energies_async(self.sim.fields, d.nx, d.ny, d.nz, d.num_ghosts)
        pic.check_status()
        return float(e.sum().item())

    # ------------------------------------------------------------ reverse
    def backward(self):
        """Reverse sweep; returns (lambda_particles dict, lambda_fields (num_cells, 9))."""
        d, p = self.deck, self.p
        nx, ny, nz, ng = d.nx, d.ny, d.nz, d.num_ghosts
        lib = capi.load()
        grid = capi.make_grid(nx, ny, nz, ng, d.boundary)
        prec = self.sim.particles.precision
        stream = torch.cuda.current_stream().cuda_stream
        status = pic.status_word()
        flags = (capi.CPIC_PUSH_TRUE_SQRT if self.true_sqrt else 0) | capi.CPIC_ADJ_INTERP_ROWS
        prm = capi.CpicPushParams(float(p["qdt_2mc"]), float(p["cdt_dx"]), float(p["cdt_dy"]),
                                  float(p["cdt_dz"]), float(p["qsp"]), prec, d.vl, flags, 0)
        h = d.R(0.5)
        hp = [float(d.R(h * p[k])) for k in ("px", "py", "pz")]
        fp = [float(p[k]) for k in ("px", "py", "pz")]
        # lambda at step K: dL/dE = E, dL/dcB = cB on the interior (ghost cells unused)
        L = self.lam_fields
        L.buf.copy_(self.sim.fields.buf)
        L.buf.view(-1, 9, 32)[:, 6:9, :] = 0
        self.lam_part.buf.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for seg in range(len(self.checkpoints) - 1, -1, -1):
            s0 = seg * self.C
            s1 = min(self.K, s0 + self.C)
            # recompute the segment, keeping per step the particles before the
            # step and the step's interpolator array (what the push adjoint
            # reads; the field transposes are linear and need no forward
            # state).  Each push writes the next step's list out of place, the
            # first reads the checkpoint's, and the last step needs only its
            # interpolator array: nothing is copied.
            ckP, ckF = self.checkpoints[seg]
            sim = self.sim
            sim.fields.buf.copy_(ckF)
            keep = (sim.particles.buf, sim.interpolators.buf)
            seg_P = [ckP] + self._seg_P
            try:
                for n in range(s0, s1):
                    sim.particles.buf = seg_P[n - s0]
                    sim.interpolators.buf = self._seg_I[n - s0]
                    last = n + 1 == s1
                    self._step(out=None if last else seg_P[n - s0 + 1], interp_only=last)
            finally:
                sim.particles.buf, sim.interpolators.buf = keep
            for n in range(s1 - 1, s0 - 1, -1):
                P, I = seg_P[n - s0], self._seg_I[n - s0]
                lib.call("cpic_adjoint_advance_b", L.ptr, *hp, C.byref(grid), prec, stream)
                lib.call("cpic_adjoint_advance_e", L.ptr, *fp, C.byref(grid), float(p["dt_eps0"]), prec, stream)
                lib.call("cpic_adjoint_advance_b", L.ptr, *hp, C.byref(grid), prec, stream)
                lib.call("cpic_adjoint_unload_accumulator", L.ptr, self.lam_acc.ptr, C.byref(grid),
                         float(p["dx"]), float(p["dy"]), float(p["dz"]), float(p["dt"]), prec, stream)
                self.lam_interp_rows.zero_()
                lib.call("cpic_adjoint_push", P.data_ptr(), d.num_particles, I.data_ptr(),
                         self.lam_acc.ptr, self.lam_part.ptr, self.lam_interp_rows.data_ptr(), C.byref(grid),
                         C.byref(prm), status.data_ptr(), stream)
                lib.call("cpic_adjoint_load_interpolator_rows", self.lam_interp_rows.data_ptr(), L.ptr,
                         C.byref(grid), prec, stream)
        torch.cuda.synchronize()
        self.timing["backward_s"] = time.perf_counter() - t0
        pic.check_status()
        return self.lam_part.download(), L.get_members()


def two_stream_drift_gradients(lam_particles: dict, deck: D.Deck, host: dict):
    """Chain rule from the initial momenta to the two-stream parameters
    (ux = sign * drift + amp * drift * sin(mode X)): returns (dL/ddrift, dL/damp)."""
    amp, mode, drift = deck.extra.get("amp", 1e-3), deck.extra.get("mode", 3), deck.v0
    X = host["X"]
    sign = host["sign"]
    lux = lam_particles["ux"].astype(np.float64)
    d_drift = np.sum(lux * (sign + amp * np.sin(mode * X)))
    d_amp = np.sum(lux * drift * np.sin(mode * X))
    return float(d_drift), float(d_amp)


def measure(case: str = "two-stream", K: int = None, checkpoint: int = 20, precision: int = 4) -> dict:
    """Forward and reverse cost of the adjoint runs of the adjoint configuration:
    two-stream 256 x 1 x 1 cells, 256 particles per cell per beam, K = 400;
    or a 64^3 thermal plasma at 16 ppc, K = 50, initial uniform E_x."""
    if case == "two-stream":
        K = K or 400
        deck = D.two_stream_1d(precision=precision, nx=256, ppc_per_beam=256, num_steps=K)
        host = D.two_stream_1d_particles(deck)
        run = AdjointRun(deck, host, checkpoint=checkpoint)
        run.forward(K)  # warm-up (kernel loading, first use of the buffers); not timed
        run.backward()
        run.reset()
        loss = run.forward(K)
        lam, _ = run.backward()
        g_drift, g_amp = two_stream_drift_gradients(lam, deck, host)
        grads = {"dL/ddrift": g_drift, "dL/damp": g_amp}
    else:
        K = K or 50
        deck = D.thermal(n=64, ppc=16, precision=precision, num_steps=K)
        f = np.zeros((deck.num_cells, 9))
        f[:, 0] = 0.01
        # particles from the seeded device loader (the host restatement's particles)
        run = AdjointRun(deck, None, fields_init=f, checkpoint=checkpoint)
        run.forward(K)  # warm-up; not timed
        run.backward()
        run.reset()
        loss = run.forward(K)
        _, lamF = run.backward()
        a = lamF.reshape(deck.nz + 2, deck.ny + 2, deck.nx + 2, 9)[1:-1, 1:-1, 1:-1]
        grads = {"dL/dE0x": float(a[..., 0].sum())}
    # the reverse sweep includes one forward recompute of every segment
    fwd, bwd = run.timing["forward_s"], run.timing["backward_s"]
    return {"case": case, "particles": deck.num_particles, "K": K, "checkpoint": checkpoint,
            "precision": precision, "loss": loss, "gradients": grads, "forward_s": fwd,
            "backward_s": bwd, "backward_over_forward": bwd / fwd}


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="two-stream", choices=["two-stream", "thermal3d"])
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--checkpoint", type=int, default=20)
    ap.add_argument("--precision", type=int, default=4)
    a = ap.parse_args()
    torch.cuda.set_device(0)
    print(json.dumps(measure(a.case, a.steps, a.checkpoint, a.precision)))
