"""Benchmark: particle pushes per second of the full PIC step on one GB300.

Workload (the reference's throughput configuration): uniform thermal plasma,
128^3 periodic cells, 64 electrons per cell (134,217,728 particles), FP32,
u_th = 0.05, dt = 0.7 Courant, zero initial fields, particles re-sorted by
cell every 20 steps (keyed by the cell each particle reaches 10 pushes later,
so that the list is in cell order midway between sorts; any order is a valid
list).  A "step" is the reference's whole time step
(example/example.cpp:221-271): interpolator load, accumulator clear, push with
deposit, accumulator unload, B half step, E step, B half step, field energies,
plus the amortised sort.  The particle list (4.3 GB) is larger than L2, so no
L2 flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  `value` is pushes/s with the state resident in HBM;
`e2e` is the same metric through the public API with the initial state copied
from pinned host memory and the final state copied back inside the timed
region (plus each step's energies read back; median of five timed runs);
`e2e_cpp` the same through the C++ push() interface; `roofline` covers the push
kernel; `cpu_baseline` is the CPU restatement (OpenMP, all host cores) on a
bounded sample of the same workload.  `--impl reference` times that CPU
implementation as the reference arm (the reference itself needs Kokkos and
Cabana, which are not available to build).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SORT_INTERVAL = 20
SORT_AHEAD = SORT_INTERVAL // 2  # sort keys: the cells this many pushes ahead
E2E_RUNS = 5  # timed end-to-end runs (after one untimed); the median is reported
N_CELLS = 128
PPC = 64
TILES = True
WORKLOAD = "thermal"
# CPU baseline: the whole workload (128^3 x 64 ppc), a bounded number of
# steps; 15 steps are about 12 s on 16 Grace cores
CPU_SAMPLE_STEPS = 15
# algorithmic bytes of push+deposit: per particle read 7 reals + cell, write 6
# reals; per interior cell the 18 interpolator coefficients and 12 accumulators
BYTES_PER_PARTICLE = {4: 56, 8: 108}
BYTES_PER_CELL = {4: 120, 8: 240}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic_from_profiles():
    """DRAM bytes per push launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "push_thermal128_fp32.md")
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(r"traffic_bytes_per_full_launch:\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        import tempfile
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        cmd = ["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits", "-lms", "200"]
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].strip()
        if vis:
            cmd += ["-i", vis]
        try:
            self.proc = subprocess.Popen(cmd, stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _barrier_max(x, ws, device="cuda"):
    """Max of a per-rank time over the ranks (the slowest replica sets the time)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, ms_per_rank, ws, device="cuda"):
    """Whole-job throughput of N independent replicas: all ranks' units over
    the slowest rank's time (units/s)."""
    if ws == 1:
        return units_per_rank / (ms_per_rank / 1e3), ms_per_rank
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(units_per_rank)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    ms = _barrier_max(ms_per_rank, ws, device)
    return float(t.item()) / (ms / 1e3), ms


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------- GPU arm
def _deck(precision, steps):
    from cabanapic_gb300 import decks
    if WORKLOAD == "diocotron":
        return decks.diocotron(precision=precision, num_steps=steps)
    return decks.thermal(n=N_CELLS, ppc=PPC, precision=precision, num_steps=steps)


def gpu_run(precision, steps, warmup, ws, host_packed=None, exact=False):
    """Device-resident timed loop; returns dict with times and push events."""
    import torch
    from cabanapic_gb300 import decks
    from cabanapic_gb300.simulation import Simulation

    deck = _deck(precision, steps + warmup)
    fields = None
    if WORKLOAD == "diocotron":
        host_packed, fields = decks.diocotron_state(deck, packed=True)
    # host_packed None: the thermal plasma is generated on the device (seeded
    # Philox, csrc/init.cu) and its initial state copied out for the other legs
    # graphs: steps that do not sort replay a captured graph of their launches
    sim = Simulation(deck, host_packed, sort_interval=SORT_INTERVAL, sort_ahead=SORT_AHEAD,
                     max_steps=steps + warmup + SORT_INTERVAL, exact=exact, tiles=TILES, fields=fields, graphs=True)
    if host_packed is None:
        host_packed = sim.particles.download_bytes()
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        sim.step()
    sim.prepare_graphs()  # both particle buffers' graphs, before the timed region
    torch.cuda.synchronize()
    _barrier(ws)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        sim.step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    # the push and the other phases, timed with events between them in one
    # more sort interval after the timed region (launched eagerly there)
    sim.time_phases = True
    steps_before = sim.step_no
    for _ in range(SORT_INTERVAL):
        sim.step()
    phases = sim.phase_times_ms()
    push_ms = [p["push"] for p in phases]
    phase_sort_steps = [k for k in range(len(phases)) if (steps_before + k) % SORT_INTERVAL == 0]
    sim.check_status()
    # timed steps that sorted first (step numbers count the warm-up steps)
    sort_steps = [k for k in range(steps) if (warmup + k) % SORT_INTERVAL == 0]
    res = dict(ms=ms, push_ms=push_ms, deck=deck, energies=sim.energies(), sort_steps=sort_steps,
               phases=phases, phase_sort_steps=phase_sort_steps)
    del sim
    torch.cuda.empty_cache()
    return res, host_packed


def _phase_summary(res, deck, peak, steps):
    """Mean CUDA-event times of the step's phases over one sort interval, the
    field phase against its algorithmic bytes (324 B per ghosted cell: interp
    96, clear 48, unload 60, 2x advance_b 72, advance_e 48) and the sort
    amortised over the sort interval."""
    ph = res["phases"]
    mean = lambda k: float(np.mean([p[k] for p in ph]))
    sorts = [p["sort"] for k, p in enumerate(ph) if k in res["phase_sort_steps"]]
    field_ms = mean("interp_clear") + mean("field_solve")
    field_bytes = 324 * deck.num_cells
    achieved = field_bytes / (field_ms / 1e3) / 1e9
    n = deck.num_particles
    # count (cell 4 B; look-ahead keys: the other 24 B of the record in, the
    # key parked in the output list 4 B out), scatter (key 4, perm 4), gather
    # in two passes (perm 2 x 4, record 32 in, 32 out)
    sb = 84 + (28 if SORT_AHEAD else 0)
    return {
        "phases_ms": {"interp_clear": mean("interp_clear"), "push": mean("push"),
                      "field_solve": mean("field_solve"),
                      "sort_amortised": float(np.sum(sorts)) / len(ph) if sorts else 0.0},
        "field_phase": {"ms": field_ms, "algorithmic_bytes": field_bytes, "achieved_gbs": achieved,
                        "frac": achieved / peak,
                        "basis": "324 B per ghosted cell: interp 96, clear 48, unload 60, 2x advance_b 72, "
                                 "advance_e 48 (energies excluded)"},
        "sort": {"ms_per_sort": float(np.mean(sorts)) if sorts else None, "sorts": len(sorts),
                 "interval": SORT_INTERVAL, "keys_ahead": SORT_AHEAD, "bytes_per_particle_per_sort": sb,
                 "achieved_gbs": (sb * n / (np.mean(sorts) / 1e3) / 1e9) if sorts else None,
                 "amortised_bytes_per_particle_per_step": sb / SORT_INTERVAL},
    }


def e2e_run(precision, steps, warmup, host_packed, ws):
    """Same step loop through the public API, with host buffers
    (Simulation.run_from_host): the initial particle state is copied from
    pinned host memory in 8 pieces, each step's energies are read back to
    pinned host memory, and the final particle state is copied back, all
    inside the timed region.  The first step's push starts on each piece as it
    lands and the last step's push hands each piece to its copy back."""
    import torch
    from cabanapic_gb300 import decks, pic
    from cabanapic_gb300.simulation import Simulation

    deck = decks.thermal(n=N_CELLS, ppc=PPC, precision=precision, num_steps=steps + warmup)
    pinned_in = torch.from_numpy(host_packed).pin_memory()
    pinned_out = torch.empty_like(pinned_in).pin_memory()
    energies_host = torch.empty((steps, 2), dtype=torch.float64).pin_memory()
    # warm-up on the same arrays (not timed), then reset the state from the host
    sim = Simulation(deck, host_packed, sort_interval=SORT_INTERVAL, sort_ahead=SORT_AHEAD,
                     max_steps=steps + warmup + SORT_INTERVAL, tiles=TILES, graphs=True)
    for _ in range(warmup):
        sim.step()
    sim.prepare_graphs()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    # One untimed pass of the whole path, then E2E_RUNS timed runs from the
    # same host state; the median is reported.  The host link is shared with
    # the rest of the machine: single copies of the list have been seen at
    # 35-190 GB/s against the usual 210 GB/s, and right after another process
    # released tens of GB of host memory the first runs took 2-2.6x longer.
    samples = []
    for rep in range(E2E_RUNS + 1):
        # the seeded list is in cell order, where look-ahead keys put a list
        # halfway through a sort interval: the run starts there (its first
        # step does not sort, so its push can start on the first pieces)
        sim.step_no = SORT_INTERVAL // 2 if SORT_AHEAD else 0
        _barrier(ws)
        e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
        e0.record(stream)
        sim.fields.buf.zero_()
        sim.run_from_host(pinned_in, steps, pinned_out, energies_host)
        e1.record(stream)
        torch.cuda.synchronize()
        if rep > 0:
            samples.append(e0.elapsed_time(e1))
    ms = float(np.median(samples))
    pic.check_status()
    # the host link's rate right after the timed region (outside it): one
    # upload and one download of the list alone
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record(stream)
    sim.particles.upload_pinned(pinned_in)
    ev[1].record(stream)
    sim.particles.download_pinned(pinned_out)
    ev[2].record(stream)
    torch.cuda.synchronize()
    link = {"h2d_gbs": host_packed.nbytes / ev[0].elapsed_time(ev[1]) / 1e6,
            "d2h_gbs": host_packed.nbytes / ev[1].elapsed_time(ev[2]) / 1e6}
    h2d = host_packed.nbytes
    d2h = host_packed.nbytes + steps * 16
    del sim
    torch.cuda.empty_cache()
    return dict(ms=ms, h2d_per_step=h2d / steps, d2h_per_step=d2h / steps, link=link, samples=samples)


# ---------------------------------------------------------------- CPU (oracle) arm
def cpu_sample_run(steps, warmup, precision=4, threads=0):
    """The CPU restatement (OpenMP push with per-thread accumulator copies,
    field phase in C++) on the workload itself (N_CELLS^3 x PPC, the same
    seeded particles, generated on the host by the oracle's OpenMP loader);
    returns (pushes/s, threads, particles, seconds)."""
    import oracle
    from cabanapic_gb300 import decks, layout as L

    orc = oracle.load()
    deck = decks.thermal(n=N_CELLS, ppc=PPC, precision=precision)
    p = deck.derived()
    R = deck.R
    buf = orc.thermal_particles(deck)
    nc = deck.num_cells
    g = orc.grid(deck.nx, deck.ny, deck.nz)
    fields = np.zeros(L.cell_array_bytes(nc, 9, R) // np.dtype(R).itemsize, R)
    interp = np.zeros(L.cell_array_bytes(nc, 18, R) // np.dtype(R).itemsize, R)
    acc = np.zeros((nc, 3, 4), R)
    n = deck.num_particles
    h = R(0.5)
    used = 1

    def one_step():
        nonlocal used
        orc.load_interpolator(fields, interp, g)
        acc.fill(0)
        used = orc.push_omp(buf, n, 32, interp, p["qdt_2mc"], p["cdt_dx"], p["cdt_dy"], p["cdt_dz"],
                            p["qsp"], acc, g, threads)
        orc.unload_accumulator(fields, acc, g, p["dx"], p["dy"], p["dz"], p["dt"])
        orc.advance_b(fields, R(h * p["px"]), R(h * p["py"]), R(h * p["pz"]), g)
        orc.advance_e(fields, p["px"], p["py"], p["pz"], g, p["dt_eps0"])
        orc.advance_b(fields, R(h * p["px"]), R(h * p["py"]), R(h * p["pz"]), g)
        orc.energies(fields, g)

    for _ in range(warmup):
        one_step()
    t0 = time.perf_counter()
    for _ in range(steps):
        one_step()
    dt = time.perf_counter() - t0
    return n * steps / dt, used, n, dt


# ---------------------------------------------------------------- main
def main():
    global N_CELLS, PPC, TILES, WORKLOAD, SORT_AHEAD, SORT_INTERVAL
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-exact", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--cells", type=int, default=N_CELLS, help="cells per axis (profiling cases)")
    ap.add_argument("--ppc", type=int, default=PPC, help="particles per cell (profiling cases)")
    ap.add_argument("--workload", default="thermal", choices=["thermal", "diocotron"],
                    help="thermal: the headline 128^3 x 64 ppc plasma; diocotron: the 96x96x64 "
                         "column at 128 ppc (heavy cell crossing), push + step timing only")
    ap.add_argument("--streaming", action="store_true",
                    help="streaming push kernel instead of the tiled one (comparison runs)")
    ap.add_argument("--sort-interval", type=int, default=SORT_INTERVAL,
                    help="steps between cell sorts (comparison runs)")
    ap.add_argument("--sort-ahead", type=int, default=None,
                    help="sort keys: the cells this many pushes ahead (default half the sort interval; "
                         "0: the current cells)")
    args = ap.parse_args()
    N_CELLS, PPC, TILES = args.cells, args.ppc, not args.streaming
    SORT_INTERVAL = max(1, args.sort_interval)
    SORT_AHEAD = SORT_INTERVAL // 2 if args.sort_ahead is None else args.sort_ahead
    WORKLOAD = args.workload
    ws, rank, local = _dist()
    metric = "particle-pushes/s (full step, FP32)"
    unit = "particle-pushes/s"
    workload = (f"thermal plasma {N_CELLS}^3 cells x {PPC} ppc = {N_CELLS ** 3 * PPC:,} particles, "
                f"FP32, u_th=0.05, dt=0.7 Courant, sort every {SORT_INTERVAL} steps on the cells {SORT_AHEAD} "
                "pushes ahead; full step (interp, clear, "
                "push+deposit, unload, advance_b/e/b, energies)")

    if args.impl == "reference":
        if rank != 0:
            return
        steps = max(1, args.steps)
        warm = max(args.warmup, 3)  # the GPU arm's warm-up
        v, cores, n, secs = cpu_sample_run(steps, warm)
        sample = (f"the workload itself: {N_CELLS}^3 grid x {PPC} ppc ({n:,} particles, the same seeded "
                  f"plasma), {steps} timed full steps after {warm} warm-up steps ({secs:.1f} s); CPU "
                  "restatement of the reference (OpenMP push with per-thread accumulator copies, field "
                  "phase in C++)")
        line = {"impl": "reference", "metric": metric, "value": v, "unit": unit, "n_gpus": args.gpus,
                "steps": steps, "warmup": warm, "ms_per_step": secs / steps * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": {"workload": workload, "sample": sample},
                "cpu_baseline": {"value": v, "unit": unit, "cores": cores, "kind": "port", "sample": sample},
                "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from cabanapic_gb300 import capi
    capi.load()

    sampler = ClockSampler()
    sampler.start()
    res, host_packed = gpu_run(4, args.steps, max(args.warmup, 3), ws)
    clocks = sampler.stop()
    deck = res["deck"]
    n = deck.num_particles
    value, ms = replica_throughput(n * args.steps, res["ms"], ws)
    push_ms = float(np.mean(res["push_ms"]))
    alg_bytes = n * BYTES_PER_PARTICLE[4] + deck.num_interior * BYTES_PER_CELL[4]
    peak, peak_kind = _peaks()
    achieved = alg_bytes / (push_ms / 1e3) / 1e9
    if WORKLOAD == "diocotron":
        if rank == 0:
            print(json.dumps({
                "metric": metric, "value": value, "unit": unit, "n_gpus": ws, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "diocotron column 96x96x64 cells, annulus 0.20<r/R<0.35 at 128 "
                                       "particles per cell of annulus volume, cB_z = 5, E x B loading "
                                       f"from the t=0 Poisson field, dt=0.99 Courant, sort every {SORT_INTERVAL} steps on "
                                       f"the cells {SORT_AHEAD} pushes ahead",
                           "particles": n, "cells": deck.num_cells,
                           "push_kernel": "tiled" if TILES else "streaming"},
                "push_ms": push_ms, "push_ms_by_step": [round(t, 4) for t in res["push_ms"]],
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "peak_kind": peak_kind,
                             "algorithmic_bytes_per_launch": alg_bytes},
                "clocks": clocks}), flush=True)
        return
    traffic = _traffic_from_profiles()
    per_step_launches = 11  # interp, push, unload, 2x(advance_b + ghost copy), fold, ghost copy, advance_e, energies
    # a sort adds count, 3 scan passes, scatter and the gather's two passes
    launches = args.steps * per_step_launches + 7 * len(res["sort_steps"])
    phases = _phase_summary(res, deck, peak, args.steps)

    exact = None
    if not args.no_exact:
        kx = max(2, min(args.steps, 20))
        rx, _ = gpu_run(4, kx, max(args.warmup, 3), ws, host_packed, exact=True)
        msx = _barrier_max(rx["ms"], ws)
        exact = {"value": n * kx * ws / (msx / 1e3), "ms_per_step": msx / kx, "steps": kx,
                 "push_ms": float(np.mean(rx["push_ms"])),
                 "note": "bit-exact push variant (unfused arithmetic, IEEE div/sqrt)"}

    e2e = None
    if not args.no_e2e:
        r = e2e_run(4, args.steps, max(args.warmup, 3), host_packed, ws)
        ems = _barrier_max(r["ms"], ws)
        e2e = {"value": n * args.steps * ws / (ems / 1e3), "unit": unit,
               "h2d_bytes_per_step": int(r["h2d_per_step"]), "d2h_bytes_per_step": int(r["d2h_per_step"]),
               "ms_per_step": ems / args.steps,
               "path": "Simulation.run_from_host (8 pieces; first push and last download overlapped)",
               "host_link_after_gbs": {k: round(v, 1) for k, v in r["link"].items()},
               "runs_ms": [round(t, 3) for t in r["samples"]], "of_runs": "median"}
    del host_packed

    e2e_cpp = None
    if not args.no_e2e and WORKLOAD == "thermal":
        # the same end-to-end measurement through the C++ push() interface
        # (include/cpic/cabana.hpp): the reference's time loop in C++, the
        # initial state uploaded from pinned host memory and the final state
        # downloaded inside the timed region, energies read back every step
        from cabanapic_gb300 import build as lib_build
        torch.cuda.empty_cache()
        cmd = [lib_build.MINIPIC, "thermal", str(N_CELLS), str(PPC), str(args.steps), str(max(args.warmup, 3)),
               str(SORT_INTERVAL)]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
        if r.returncode == 0:
            d = json.loads(r.stdout.strip().splitlines()[-1])
            e2e_cpp = {"value": d["pushes_per_s"], "unit": unit, "ms_per_step": d["ms"] / d["steps"],
                       "h2d_bytes_per_step": d["h2d_bytes"] // d["steps"],
                       "d2h_bytes_per_step": d["d2h_bytes"] // d["steps"], "path": d["path"],
                       "runs_ms": d.get("runs_ms"), "of_runs": "median"}
        else:
            e2e_cpp = {"error": (r.stderr or r.stdout).strip()[-300:]}

    fp64 = None
    if not args.no_fp64:
        k64 = max(2, min(args.steps, 10))
        r64, hp = gpu_run(8, k64, 3, ws)
        del hp
        ms64 = _barrier_max(r64["ms"], ws)
        p64 = float(np.mean(r64["push_ms"]))
        fp64 = {"value": n * k64 * ws / (ms64 / 1e3), "ms_per_step": ms64 / k64, "steps": k64,
                "push_ms": p64, "fp32_over_fp64": (value / (n * k64 * ws / (ms64 / 1e3)))}

    adjoint = None
    if not args.no_adjoint:
        # the adjoint configuration's two cases: forward K steps with
        # checkpoints, then the reverse sweep (segment recompute + transposed
        # steps); wall clock after a warm-up pair of passes
        from cabanapic_gb300 import adjoint as adj
        adjoint = {}
        for case in ("two-stream", "thermal3d"):
            r = adj.measure(case)
            adjoint[case] = {k: r[k] for k in ("particles", "K", "checkpoint", "forward_s", "backward_s",
                                               "backward_over_forward", "gradients")}
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and not args.no_cpu:
        v, cores, ns, secs = cpu_sample_run(CPU_SAMPLE_STEPS, 1)
        cpu = {"value": v, "unit": unit, "cores": cores, "kind": "port",
               "sample": f"the workload itself ({N_CELLS}^3 grid x {PPC} ppc, {ns:,} particles), "
                         f"{CPU_SAMPLE_STEPS} full steps after 1 ({secs:.1f} s)"}

    if rank == 0:
        line = {
            "metric": metric, "value": value, "unit": unit, "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload, "particles": n, "cells": deck.num_cells,
                       "l2": f"particle list {n * 32 / 1e9:.2f} GB > 129 MB L2: no flush needed",
                       "replicas": ws, "push_kernel": "tiled" if TILES else "streaming",
                       "seed": int(deck.extra.get("seed", 2024)),
                       "rng": "Philox4x32-10 keyed by particle index, generated on the device"},
            "push_ms": push_ms,
            "push_ms_by_step": [round(t, 4) for t in res["push_ms"]],
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": alg_bytes},
            "clocks": clocks, "e2e": e2e, "e2e_cpp": e2e_cpp, "gpu_launches": launches, "fp64": fp64, "exact": exact,
            "phases_ms": phases["phases_ms"], "field_phase": phases["field_phase"], "sort": phases["sort"],
            "cpu_baseline": cpu,
            "adjoint": adjoint,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
