"""Precision study against the FP64 oracle (verification harness, not collected
by pytest): the thermal plasma of the precision configuration (128^3 cells x
32 ppc = 67,108,864 particles, 1000 steps, seed 2024) run in lockstep by

  (a) the FP32 GPU path (FP32 push, deposit and field stencils; FP64 energy
      and charge reductions), sorted by cell every 20 steps;
  (b) the full-FP64 GPU build, same schedule;
  (c) the FP64 oracle: the reference's step sequence (example/example.cpp:
      221-266) with real_t = double and its literal sqrtf (src/push.h:148,169),
      OpenMP over particles on the host cores -- the reference built with
      real_t = double, restated.

All three start from the same particles: the seeded device loader's FP64
list, rounded to FP32 for (a).  Every step reports the field L2 relative
error ||F - F_c|| / ||F_c|| over E and cB on the interior and the field-energy
error |W - W_c| / W_c of (a) and (b) against (c); every `--sample` steps the
total-energy drift of each run (field + kinetic, relative to step 0) and the
charge residual max |(div E - rho/eps0)(t) - (...)(0)| / max |rho/eps0| of the
GPU runs (the oracle's at the last step only: a numpy restatement, slow at
this size).  Prints one JSON object.

    python tests/precision_vs_oracle.py [--cells 128] [--ppc 32] [--steps 1000]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def main():
    import torch

    import oracle
    from oracle import diagnostics as od
    from cabanapic_gb300 import decks as D, layout as L
    from cabanapic_gb300.precision import _Tracker, _interior_fields
    from cabanapic_gb300.simulation import Simulation

    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=128)
    ap.add_argument("--ppc", type=int, default=32)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--sample", type=int, default=50)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--out", default=None, help="also write the JSON here")
    a = ap.parse_args()
    torch.cuda.set_device(0)
    orc = oracle.load()

    n = a.cells
    deck64 = D.thermal(n=n, ppc=a.ppc, precision=8, num_steps=a.steps, seed=a.seed)
    deck32 = D.thermal(n=n, ppc=a.ppc, precision=4, num_steps=a.steps, seed=a.seed)
    host64 = D.thermal_particles_device(deck64, device="cuda").download()
    host32 = {k: (v.astype(np.float32) if k != "cell" else v) for k, v in host64.items()}
    host32["w"] = np.full(len(host32["w"]), deck32.derived()["we"], np.float32)
    sims = {"fp32": Simulation(deck32, host32, sort_interval=20, max_steps=a.steps),
            "fp64": Simulation(deck64, host64, sort_interval=20, max_steps=a.steps)}
    trk = {k: _Tracker(s) for k, s in sims.items()}

    # the oracle's state
    p = deck64.derived()
    nc = deck64.num_cells
    g = orc.grid(n, n, n)
    buf = L.pack_particles(host64, np.float64, 32)
    del host64, host32
    fields = np.zeros(L.cell_array_bytes(nc, 9, np.float64) // 8, np.float64)
    interp = np.zeros(L.cell_array_bytes(nc, 18, np.float64) // 8, np.float64)
    acc = np.zeros((nc, 3, 4), np.float64)
    h = 0.5
    dV = float(p["dx"] * p["dy"] * p["dz"])

    def oracle_fields():
        return L.unpack_cells(fields, nc, 9)[:, :6].reshape(n + 2, n + 2, n + 2, 6)[1:-1, 1:-1, 1:-1]

    def oracle_total():
        parts = L.unpack_particles(buf, deck64.num_particles, np.float64, 32)
        e = orc.energies(fields, g)
        return float((e[2] + e[3]) * dV + od.kinetic_energy(parts))

    def oracle_charge():
        parts = L.unpack_particles(buf, deck64.num_particles, np.float64, 32)
        rho = od.charge_density(parts, n, n, n, float(p["qsp"]), float(p["dx"]), float(p["dy"]), float(p["dz"]))
        r = od.gauss_residual(L.unpack_cells(fields, nc, 9), rho, n, n, n, float(p["dx"]), float(p["dy"]),
                              float(p["dz"]), float(p["eps"]))
        return r, float(np.abs(rho).max() / float(p["eps"]))

    e_orc0 = oracle_total()
    r_orc0, rho_max = oracle_charge()
    rows = []
    t_orc = 0.0
    for step in range(1, a.steps + 1):
        for s in sims.values():
            s.step()
        t0 = time.perf_counter()
        orc.load_interpolator(fields, interp, g)
        acc.fill(0)
        orc.push_omp(buf, deck64.num_particles, 32, interp, p["qdt_2mc"], p["cdt_dx"], p["cdt_dy"],
                     p["cdt_dz"], p["qsp"], acc, g)
        orc.unload_accumulator(fields, acc, g, p["dx"], p["dy"], p["dz"], p["dt"])
        orc.advance_b(fields, h * p["px"], h * p["py"], h * p["pz"], g)
        orc.advance_e(fields, p["px"], p["py"], p["pz"], g, p["dt_eps0"])
        orc.advance_b(fields, h * p["px"], h * p["py"], h * p["pz"], g)
        w_orc = float(orc.energies(fields, g)[2:4].sum())
        t_orc += time.perf_counter() - t0
        fc = torch.from_numpy(np.ascontiguousarray(oracle_fields()))
        nrm = float(torch.linalg.vector_norm(fc))
        row = {"step": step, "w_oracle": w_orc}
        for k, s in sims.items():
            f = _interior_fields(s).cpu()
            row[f"field_l2_rel_{k}"] = float(torch.linalg.vector_norm(f - fc)) / nrm if nrm > 0 else 0.0
            w = float(s.energy[step - 1].sum().item())
            row[f"w_{k}"] = w
            row[f"field_energy_rel_err_{k}"] = abs(w - w_orc) / w_orc if w_orc > 0 else 0.0
        if step % a.sample == 0 or step == a.steps:
            for k in sims:
                row[f"energy_drift_{k}"] = (trk[k].total_energy() - trk[k].e0) / trk[k].e0
                row[f"charge_err_{k}"] = trk[k].charge_error()
            row["energy_drift_oracle"] = (oracle_total() - e_orc0) / e_orc0
            if step == a.steps:
                r, _ = oracle_charge()
                row["charge_err_oracle"] = float(np.abs(r - r_orc0).max()) / rho_max
        rows.append(row)
        if step % 100 == 0:
            print(json.dumps(row), file=sys.stderr, flush=True)
    for s in sims.values():
        s.check_status()

    def mx(key):
        return max(r[key] for r in rows)

    half = rows[len(rows) // 2:]
    w_or = np.mean([r["w_oracle"] for r in half])
    out = {
        "config": f"thermal plasma {n}^3 x {a.ppc} ppc = {deck64.num_particles:,} particles, {a.steps} steps, "
                  f"seed {a.seed}; GPU runs sorted every 20 steps; oracle FP64 with literal sqrtf, OpenMP",
        "oracle_threads": orc.num_threads(), "oracle_s_per_step": t_orc / a.steps,
        "max_field_l2_rel_fp32": mx("field_l2_rel_fp32"), "max_field_l2_rel_fp64": mx("field_l2_rel_fp64"),
        "max_field_energy_rel_err_fp32": mx("field_energy_rel_err_fp32"),
        "max_field_energy_rel_err_fp64": mx("field_energy_rel_err_fp64"),
        "field_energy_level_rel_diff_second_half_fp32": abs(np.mean([r["w_fp32"] for r in half]) - w_or) / w_or,
        "field_energy_level_rel_diff_second_half_fp64": abs(np.mean([r["w_fp64"] for r in half]) - w_or) / w_or,
        "final": rows[-1],
        "rows_sampled": [r for r in rows if r["step"] % a.sample == 0],
        "rows_early": rows[:10],
    }
    s = json.dumps(out)
    print(s)
    if a.out:
        with open(a.out, "w") as fh:
            fh.write(s + "\n")


if __name__ == "__main__":
    main()
