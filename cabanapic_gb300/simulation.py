"""Time-loop driver: the per-step sequence of the reference's main()
(example/example.cpp:216-271) on one GPU, through the C ABI.

Each step: load_interpolator_array -> clear_accumulator_array -> [cell sort
every `sort_interval` steps, keyed by the cells `sort_ahead` pushes ahead
(default half the interval)] -> push -> unload_accumulator_array -> advance_b(1/2)
-> advance_e -> advance_b(1/2) -> field energies (double, kept on the device).
Energies are copied to the host on request.  With particle_dump / field_dump
(open text files) the loop also writes the reference's per-step dumps
(example.cpp:131-132, 273-277): each step's values are copied to pinned host
memory asynchronously and written at the next step (or by flush_dumps()), so
the copies overlap the following step's kernels.  With graphs=True, a step
that does not sort replays a CUDA graph of its launches (captured once per
particle buffer), removing the host launch overhead between the field phase's
small kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from . import decks as D
from . import pic
from . import layout as L
from .arrays import AccumulatorArray, FieldArray, InterpolatorArray, ParticleList, block_pieces, copy_streams


class Simulation:
    def __init__(self, deck: D.Deck, particles=None, *, device=None, sort_interval: int = 0,
                 sort_ahead: int = None, max_steps: int = None, time_push: bool = False, exact: bool = False,
                 tiles: bool = True, fields=None, particle_dump=None, field_dump=None,
                 acc_f64: bool = False, graphs: bool = False):
        self.deck = deck
        self.p = deck.derived()
        dev = torch.device(device if device is not None else "cuda")
        self.device = dev
        R = deck.R
        nc = deck.num_cells
        self.particles = ParticleList(deck.num_particles, R, deck.vl, dev)
        self.interpolators = InterpolatorArray(nc, R, dev)
        # acc_f64 (FP32 decks): FP64 accumulator rows, the compensated per-cell current sum
        self.accumulators = AccumulatorArray(nc, np.float64 if acc_f64 else R, dev)
        self.fields = FieldArray(nc, R, dev)
        self.solver = pic.EMFieldSolver(self.fields, deck.boundary)
        pic.initialize_interpolator(self.interpolators)
        if particles is None and D.is_thermal(deck):
            D.thermal_particles_device(deck, self.particles)  # seeded, generated in HBM
        else:
            if particles is None:
                particles = D.initial_particles(deck)
            self.particles.upload(particles)
        if fields is None:
            fields = D.initial_fields(deck)
        if fields is not None:
            self.fields.set_members(np.asarray(fields))
        self.sort_interval = int(sort_interval)
        # look-ahead sort keys: by default the cells half a sort interval ahead
        if self.sort_interval > 0:
            self.sort_ahead = self.sort_interval // 2 if sort_ahead is None else int(sort_ahead)
            self.sorter = pic.Sorter(self.particles, nc, double_buffer=True, steps_ahead=self.sort_ahead,
                                     ahead=((deck.nx, deck.ny, deck.nz),
                                            (self.p["cdt_dx"], self.p["cdt_dy"], self.p["cdt_dz"])))
        else:
            self.sort_ahead = 0
            self.sorter = None
        cap = max_steps if max_steps is not None else max(deck.num_steps, 1)
        self.energy = torch.zeros((cap, 2), dtype=torch.float64, device=dev)
        self.step_no = 0
        self.time_push = time_push
        self.push_events = []
        self.time_phases = False  # events between the step's phases (phase_times_ms)
        self.phase_events = []
        # graphs: a step that does not sort (and records no timing events and
        # writes no dumps) replays a CUDA graph of its kernel launches, one
        # graph per particle buffer (the sort alternates two); energies go
        # to a fixed staging slot and are copied into the history
        self.graphs = bool(graphs)
        self._graphs = {}
        self._warm = False  # one step launched eagerly (first-use setup done)
        self._e_stage = torch.zeros(2, dtype=torch.float64, device=dev)
        self.exact = bool(exact)
        self.tiles = bool(tiles)
        self.particle_dump = particle_dump
        self.field_dump = field_dump
        self._pdump = pic.ParticleDump(self.particles) if particle_dump is not None else None
        self._fdump = pic.FieldDump(self.fields, deck.nx) if field_dump is not None else None
        self._pending_step = None
        if self._pdump is not None:
            p = self.p
            particle_dump.write("#step=0\n0 ")
            self._pdump.enqueue(self.particles, 0, p["dx"], deck.nx, deck.ny, deck.nz, deck.num_ghosts,
                                deck.boundary)
            self._pdump.write(particle_dump)

    # ------------------------------------------------------------------
    def step(self) -> None:
        d, p = self.deck, self.p
        nx, ny, nz, ng = d.nx, d.ny, d.nz, d.num_ghosts
        sorted_now = self.sorter is not None and self.step_no % self.sort_interval == 0
        dumps = self._pdump is not None or self._fdump is not None
        if (self.graphs and self._warm and not sorted_now and not dumps and not self.time_push
                and not self.time_phases):
            self._graph(self.particles.buf).replay()
            if self.step_no < self.energy.shape[0]:
                self.energy[self.step_no].copy_(self._e_stage)
        else:
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)] if self.time_phases else None
            out = self.energy[self.step_no] if self.step_no < self.energy.shape[0] else None
            self._launch_step(sorted_now, ev, out)
            self._warm = True
            if ev:
                self.phase_events.append((ev, sorted_now))
        if dumps:
            self.flush_dumps()
            if self._fdump is not None:
                self._fdump.enqueue(self.fields, 0, p["dx"], nx, ny, nz, ng, d.boundary)
            if self._pdump is not None:
                self._pdump.enqueue(self.particles, 0, p["dx"], nx, ny, nz, ng, d.boundary)
            self._pending_step = self.step_no + 1  # the reference's loop counts steps from 1
        self.step_no += 1

    def _launch_step(self, sorted_now: bool, ev, energy_out, pieces=None) -> None:
        """The step's launches on the current stream (ev: 5 events between the
        phases, or None; energy_out: the energies' device slot, or None).
        pieces: push the list as runs [(start, count, before, after)] of whole
        AoSoA blocks, calling before() ahead of each run's push and after()
        behind it (stream hooks for overlapped host copies)."""
        d, p = self.deck, self.p
        nx, ny, nz, ng = d.nx, d.ny, d.nz, d.num_ghosts
        if ev:
            ev[0].record()
        pic.load_interpolator_array(self.fields, self.interpolators, nx, ny, nz, ng, boundary=d.boundary)
        pic.clear_accumulator_array(self.fields, self.accumulators, nx, ny, nz)
        if ev:
            ev[1].record()
        if sorted_now:
            self.sorter(self.particles)
        if ev:
            ev[2].record()
        if self.time_push and not ev:
            ev_push = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev_push[0].record()
        for start, count, before, after in (pieces or [(0, self.particles.n, None, None)]):
            if before is not None:
                before()
            part = self.particles if pieces is None else self.particles.view(start, count)
            pic.push(part, self.interpolators, p["qdt_2mc"], p["cdt_dx"], p["cdt_dy"], p["cdt_dz"],
                     p["qsp"], self.accumulators, None, nx, ny, nz, ng, d.boundary, exact=self.exact,
                     tiles=self.tiles)
            if after is not None:
                after()
        if ev:
            ev[3].record()
            if self.time_push:
                self.push_events.append((ev[2], ev[3]))
        elif self.time_push:
            ev_push[1].record()
            self.push_events.append(ev_push)
        pic.unload_accumulator_array(self.fields, self.accumulators, nx, ny, nz, ng,
                                     p["dx"], p["dy"], p["dz"], p["dt"], boundary=d.boundary)
        half = d.R(0.5)
        hpx, hpy, hpz = d.R(half * p["px"]), d.R(half * p["py"]), d.R(half * p["pz"])
        self.solver.advance_b(self.fields, hpx, hpy, hpz, nx, ny, nz, ng)
        self.solver.advance_e(self.fields, p["px"], p["py"], p["pz"], nx, ny, nz, ng, p["dt_eps0"])
        self.solver.advance_b(self.fields, hpx, hpy, hpz, nx, ny, nz, ng)
        if energy_out is not None:
            self.solver.energies_async(self.fields, nx, ny, nz, ng, out=energy_out)
        if ev:
            ev[4].record()

    def _graph(self, buf: torch.Tensor):
        """The CUDA graph of a non-sorting step on particle buffer `buf`
        (captured on first use; capturing launches nothing)."""
        g = self._graphs.get(buf.data_ptr())
        if g is None:
            # first-use setup (shared-memory opt-in, occupancy, scratch)
            # happens outside the capture, in an eager step
            if not self._warm:
                raise RuntimeError("graphs are captured after one eager step")
            keep = self.particles.buf
            self.particles.buf = buf
            g = torch.cuda.CUDAGraph()
            try:
                with torch.cuda.graph(g):
                    self._launch_step(False, None, self._e_stage)
            finally:
                self.particles.buf = keep
            self._graphs[buf.data_ptr()] = g
        return g

    def reset_graphs(self) -> None:
        """Drops the captured step graphs (they hold the launch configuration:
        call this after changing exact, tiles or the arrays' buffers)."""
        self._graphs = {}

    def prepare_graphs(self) -> None:
        """Captures the step graphs of both particle buffers now (nothing is
        launched), so that no capture happens inside a timed loop."""
        if not self.graphs:
            return
        bufs = [self.particles.buf] + ([self.sorter.spare] if self.sorter is not None else [])
        for b in bufs:
            self._graph(b)

    def flush_dumps(self) -> None:
        """Writes the dumps enqueued at the last step (waits for their copies)."""
        k = self._pending_step
        if k is None:
            return
        if self._fdump is not None:
            self.field_dump.write(f"#step={k}\n")
            self._fdump.write(self.field_dump)
        if self._pdump is not None:
            t = float(self.deck.R(self.deck.R(k) * self.p["dt"]))
            self.particle_dump.write(f"#step={k}\n{t:e} ")
            self._pdump.write(self.particle_dump)
        self._pending_step = None

    def run(self, steps: int) -> None:
        for _ in range(steps):
            self.step()

    def run_from_host(self, pinned_in: torch.Tensor, steps: int, pinned_out: torch.Tensor = None,
                      energies_out: torch.Tensor = None, pieces: int = 8) -> None:
        """Uploads the particle list from pinned host memory (its AoSoA bytes),
        runs `steps` steps and, with pinned_out, downloads the final list; each
        step's energies go to energies_out (pinned [steps, 2] double) if given.
        Everything is ordered on the current stream: synchronise it before
        reading the host buffers.

        The list moves in `pieces` runs of whole AoSoA blocks on side streams.
        Unless the first step sorts (a sort needs the whole list), its push
        takes each run as soon as that run has landed; the last step's push
        hands each run to its copy back as soon as it has pushed it.  Only the
        order of the accumulator sums differs from upload, run, download."""
        if steps < 1:
            raise ValueError("steps must be >= 1")
        nbytes = self.particles.nbytes
        for name, t in (("pinned_in", pinned_in), ("pinned_out", pinned_out)):
            if t is None:
                continue
            if t.dtype != torch.uint8 or t.device.type != "cpu" or not t.is_pinned() or t.numel() < nbytes:
                raise ValueError(f"{name}: a pinned host uint8 tensor of at least {nbytes} bytes")
        if pinned_in is None:
            raise ValueError("pinned_in is required")
        if energies_out is not None and (energies_out.device.type != "cpu" or tuple(energies_out.shape[1:]) != (2,)
                                         or energies_out.shape[0] < steps):
            raise ValueError("energies_out: a host tensor of shape [steps, 2]")
        dev = self.particles.buf.device
        cur = torch.cuda.current_stream(dev)
        runs = block_pieces(self.particles.n, self.particles.vl, pieces)
        streams = copy_streams(dev, len(runs))
        blk = L.particle_block_bytes(self.particles.real, self.particles.vl)
        sorts_first = self.sorter is not None and self.step_no % self.sort_interval == 0
        if self._pdump is not None or self._fdump is not None or self.time_phases or self.time_push:
            # dumps and timing events take the plain path: upload, steps, download
            self.particles.upload_pinned(pinned_in, pieces)
            for k in range(steps):
                self.step()
                if energies_out is not None and self.step_no - 1 < self.energy.shape[0]:
                    energies_out[k].copy_(self.energy[self.step_no - 1], non_blocking=True)
            if pinned_out is not None:
                self.particles.download_pinned(pinned_out, pieces)
            return
        if sorts_first:
            self.particles.upload_pinned(pinned_in, pieces)
            up = None
        else:
            up = []
            ready = torch.cuda.Event()
            ready.record(cur)
            for (start, count), st in zip(runs, streams):
                a, b = (start // self.particles.vl) * blk, L.particle_list_bytes(start + count, self.particles.real,
                                                                                 self.particles.vl)
                st.wait_event(ready)
                with torch.cuda.stream(st):
                    self.particles.buf[a:b].copy_(pinned_in[a:b], non_blocking=True)
                self.particles.buf.record_stream(st)
                done = torch.cuda.Event()
                done.record(st)
                up.append(done)

        def download_hooks():
            hooks = []
            for (start, count), st in zip(runs, streams):
                def after(start=start, count=count, st=st):
                    a = (start // self.particles.vl) * blk
                    b = L.particle_list_bytes(start + count, self.particles.real, self.particles.vl)
                    pushed = torch.cuda.Event()
                    pushed.record(cur)
                    st.wait_event(pushed)
                    buf = self.particles.buf  # the list's buffer after this step's sort
                    with torch.cuda.stream(st):
                        pinned_out[a:b].copy_(buf[a:b], non_blocking=True)
                    buf.record_stream(st)
                hooks.append(after)
            return hooks

        for k in range(steps):
            last = k == steps - 1
            special = (k == 0 and up is not None) or (last and pinned_out is not None)
            if not special:
                self.step()
            else:
                before = [(lambda e=e: cur.wait_event(e)) for e in up] if (k == 0 and up is not None) \
                    else [None] * len(runs)
                after = download_hooks() if (last and pinned_out is not None) else [None] * len(runs)
                sorted_now = self.sorter is not None and self.step_no % self.sort_interval == 0
                out = self.energy[self.step_no] if self.step_no < self.energy.shape[0] else None
                self._launch_step(sorted_now, None, out,
                                  pieces=[(s0, c0, bf, af) for (s0, c0), bf, af in zip(runs, before, after)])
                self._warm = True
                self.step_no += 1
            if energies_out is not None and self.step_no - 1 < self.energy.shape[0]:
                energies_out[k].copy_(self.energy[self.step_no - 1], non_blocking=True)
        if pinned_out is not None:
            for st in streams:
                done = torch.cuda.Event()
                done.record(st)
                cur.wait_event(done)

    # ------------------------------------------------------------------
    def energies(self) -> np.ndarray:
        """[steps, 2] history of (E, B) field energies, accumulated in double."""
        return self.energy[: min(self.step_no, self.energy.shape[0])].cpu().numpy()

    def phase_times_ms(self) -> list:
        """Per timed step: {"interp_clear", "sort" (0 when the step did not
        sort), "push", "field_solve" (unload, advance_b/e/b, energies)} in ms."""
        torch.cuda.synchronize()
        out = []
        for ev, sorted_now in self.phase_events:
            out.append({"interp_clear": ev[0].elapsed_time(ev[1]),
                        "sort": ev[1].elapsed_time(ev[2]) if sorted_now else 0.0,
                        "push": ev[2].elapsed_time(ev[3]), "field_solve": ev[3].elapsed_time(ev[4])})
        return out

    def push_times_ms(self) -> list:
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in self.push_events]

    def check_status(self) -> None:
        pic.check_status()

    def download_particles(self) -> dict:
        return self.particles.download()
