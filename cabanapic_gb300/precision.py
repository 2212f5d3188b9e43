"""Precision study: FP32 against FP64 on the same seeded thermal plasma.

Runs (a) the FP32 path (FP32 push, deposit and field stencils; FP64 energy
and charge reductions), (a') the same with FP64 accumulator rows (the
compensated per-cell current sum) and (b) the full-FP64 GPU build from the
same initial state (drawn in FP64; (a) starts from it rounded to FP32), and
reports per step:
  * field L2 relative error of (a) against (b): ||F_a - F_b|| / ||F_b|| over
    E and cB on the interior,
  * total-energy drift of each run: field energy (0.5 sum (E^2 + cB^2) dV,
    dV = dx dy dz) plus kinetic energy (sum w m c^2 (gamma - 1)), relative to
    step 0,
  * the charge-conservation residual max |(div E - rho/eps0)(t) - (...)(0)|
    relative to max |rho/eps0|,
  * the field-energy error |W_a - W_b| / W_b of (a) against (b), W = 0.5 sum
    (E^2 + cB^2) per step (the dump_energies quantity), its maximum over the
    run, and the relative difference of the time averages over the second half
    (a thermal plasma's field energy is a fluctuation level: once the two runs
    decorrelate, the per-step values differ by the fluctuation itself while
    the level agrees),
and the pushes/s of (a) and (b).  The FP64 GPU build is the same arithmetic
as the reference built with real_t = double; the tests check the two agree
to round-off on short runs (tests/test_precision_gpu.py).

    python -m cabanapic_gb300.precision [--cells 128] [--ppc 32] [--steps 1000]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import decks as D
from . import layout as L
from . import pic
from .simulation import Simulation


def _interior_fields(sim) -> torch.Tensor:
    """E and cB on the interior as a (6, nz, ny, nx) double tensor."""
    d = sim.deck
    nc = d.num_cells
    nb = -(-nc // 32)
    a = sim.fields.buf.view(nb, 9, 32).permute(0, 2, 1).reshape(nb * 32, 9)[:nc, :6]
    a = a.reshape(d.nz + 2, d.ny + 2, d.nx + 2, 6)[1:-1, 1:-1, 1:-1].double()
    return a


class _Tracker:
    def __init__(self, sim):
        self.sim = sim
        d, p = sim.deck, sim.p
        self.diag = pic.Diagnostics(d.num_cells)
        self.args = (d.nx, d.ny, d.nz, d.num_ghosts)
        self.dxyz = (float(p["dx"]), float(p["dy"]), float(p["dz"]))
        self.dV = self.dxyz[0] * self.dxyz[1] * self.dxyz[2]
        self.qsp, self.eps, self.mc2 = float(p["qsp"]), float(p["eps"]), float(p["me"]) * float(p["c"]) ** 2
        rho = self.diag.charge_density(sim.particles, *self.args, self.qsp, *self.dxyz)
        self.r0 = torch.zeros(d.num_cells, dtype=torch.float64, device=sim.device)
        self.diag.gauss_residual(sim.fields, rho, *self.args, *self.dxyz, eps0=self.eps, resid=self.r0)
        self.rho_max = float((rho.abs() / self.eps).max())
        self.e0 = self.total_energy()

    def total_energy(self) -> float:
        s = self.sim
        d = s.deck
        fe = s.solver.energies_async(s.fields, d.nx, d.ny, d.nz, d.num_ghosts).clone()
        ke = self.diag.kinetic_energy(s.particles, self.mc2)
        return float((fe.sum() * self.dV + ke[0]).item())

    def charge_error(self) -> float:
        s = self.sim
        rho = self.diag.charge_density(s.particles, *self.args, self.qsp, *self.dxyz)
        out = self.diag.gauss_residual(s.fields, rho, *self.args, *self.dxyz, eps0=self.eps, ref=self.r0)
        return float(out[0].item()) / self.rho_max


def run(cells=128, ppc=32, steps=1000, seed=2024, sample_every=1, sort_interval=20) -> dict:
    deck64 = D.thermal(n=cells, ppc=ppc, precision=8, num_steps=steps, seed=seed)
    deck32 = D.thermal(n=cells, ppc=ppc, precision=4, num_steps=steps, seed=seed)
    host64 = D.thermal_particles_device(deck64, device="cuda").download()  # seeded, generated in HBM
    host32 = {k: (v.astype(np.float32) if k != "cell" else v) for k, v in host64.items()}
    host32["w"] = np.full(len(host32["w"]), deck32.derived()["we"], np.float32)
    sims = {"fp32": Simulation(deck32, host32, sort_interval=sort_interval, max_steps=steps),
            "fp32_acc64": Simulation(deck32, host32, sort_interval=sort_interval, max_steps=steps,
                                     acc_f64=True),
            "fp64": Simulation(deck64, host64, sort_interval=sort_interval, max_steps=steps)}
    trk = {k: _Tracker(s) for k, s in sims.items()}
    rows = []
    times = {k: 0.0 for k in sims}
    for step in range(1, steps + 1):
        for k, s in sims.items():
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.step()
            torch.cuda.synchronize()
            times[k] += time.perf_counter() - t0
        if step % sample_every == 0 or step == steps:
            fa, fb = _interior_fields(sims["fp32"]), _interior_fields(sims["fp64"])
            nb = float(torch.linalg.vector_norm(fb))
            l2 = float(torch.linalg.vector_norm(fa - fb)) / nb if nb > 0 else 0.0
            row = {"step": step, "field_l2_rel": l2}
            for k in sims:
                row[f"energy_drift_{k}"] = (trk[k].total_energy() - trk[k].e0) / trk[k].e0
                row[f"charge_err_{k}"] = trk[k].charge_error()
            rows.append(row)
    for s in sims.values():
        s.check_status()
    w32 = sims["fp32"].energies().sum(axis=1)
    w64 = sims["fp64"].energies().sum(axis=1)
    werr = np.abs(w32 - w64) / np.where(w64 > 0, w64, 1.0)
    w3264 = sims["fp32_acc64"].energies().sum(axis=1)
    werr_acc64 = np.abs(w3264 - w64) / np.where(w64 > 0, w64, 1.0)
    half = slice(len(w64) // 2, None)
    level = abs(float(w32[half].mean()) - float(w64[half].mean())) / float(w64[half].mean())
    first_1e4 = next((i + 1 for i, e in enumerate(werr) if e > 1e-4), None)
    n = deck32.num_particles
    return {
        "config": f"thermal plasma {cells}^3 x {ppc} ppc = {n:,} particles, {steps} steps, seed {seed}",
        "pushes_per_s_fp32": n * steps / times["fp32"],
        "pushes_per_s_fp64": n * steps / times["fp64"],
        "fp32_over_fp64": times["fp64"] / times["fp32"],
        "max_field_l2_rel": max(r["field_l2_rel"] for r in rows),
        "field_energy_rel_err_max": float(werr.max()),
        "field_energy_rel_err_max_fp32_acc64": float(werr_acc64.max()),
        "pushes_per_s_fp32_acc64": n * steps / times["fp32_acc64"],
        "field_energy_rel_err_final": float(werr[-1]),
        "field_energy_first_step_above_1e-4": first_1e4,
        "field_energy_level_rel_diff_second_half": level,
        "final": rows[-1],
        "rows": rows,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=128)
    ap.add_argument("--ppc", type=int, default=32)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--sample-every", type=int, default=10)
    ap.add_argument("--rows", action="store_true", help="print every sampled row")
    args = ap.parse_args()
    torch.cuda.set_device(0)
    out = run(args.cells, args.ppc, args.steps, sample_every=args.sample_every)
    if not args.rows:
        out["rows"] = out["rows"][:: max(1, len(out["rows"]) // 20)]
    print(json.dumps(out))


if __name__ == "__main__":
    main()
