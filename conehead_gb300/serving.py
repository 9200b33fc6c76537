"""Continuous-batching dose server on one GPU.

Dose requests (a phantom already resident on the device, 1..n beams and a
settings dict) arrive at any time.  The scheduler:

* splits its HBM budget (80% of the device by default) into fixed memory
  (resident phantoms, each slot's kernel tables and stencils), one scratch
  pool per slot of ``scratch_cap`` bytes, and dose outputs;
* admits requests first in, first out, while the outputs of admitted
  requests fit the rest of the budget; a request whose outputs cannot fit
  even on an idle server, or whose single beam needs more scratch than a
  slot's pool, is refused;
* keeps a queue of admitted beams and, whenever a slot is free, sends the
  oldest ones that share a voxel spacing and spectrum to the GPU as one
  ``ch_dose_batch`` call (every beam's prologue, then one persistent cone
  launch over all of them), cut down until the slot's scratch arena fits
  its pool -- one beam always fits, so admitted work never deadlocks;
* runs each slot -- a plan with its own CUDA stream -- independently, so a
  batch launched while another is on the GPU overlaps it, and requests that
  arrive meanwhile join the next batch instead of waiting for a queue to
  drain;
* hands a request back when its last beam is done: dose arrays copied to
  pinned host memory (or left on the device), with arrival, admission and
  completion times for latency statistics.

The reference computes one beam per blocking ``Conehead.calculate`` call
(conehead/conehead.py:522-738) and has no serving layer; the physics of each
beam is unchanged here, so a request's result is the same alone and in any
mix, up to the float rounding of the dose accumulation order.

``DoseServer`` talks to an executor through a small interface, so its
admission and batching logic runs on the CPU in tests with a simulated
executor; ``GpuExecutor`` is the real one.

Latency in practice: call ``GpuExecutor.warm`` once after ``prepare`` (no
request then pays for growing a slot's scratch arena -- cudaFree waits for
the whole device -- or for a first pinned host allocation), and have a
long-running server process ``gc.collect(); gc.freeze()`` after start-up,
so that the cyclic garbage collector does not walk every object the process
holds while requests are in flight.
"""
import time
import types
from collections import deque

import numpy as np


class Request:
    """One dose request.  ``beams`` is a list of (source, block) pairs."""

    _next_id = 0

    def __init__(self, phantom, beams, settings):
        self.rid = Request._next_id
        Request._next_id += 1
        self.phantom = phantom
        self.beams = list(beams)
        self.settings = settings
        self.doses = [None] * len(self.beams)
        self.t_submit = self.t_admit = self.t_launch = self.t_done = None
        self.error = None
        self.remaining = len(self.beams)
        self.reserved = 0

    @property
    def done(self):
        return self.t_done is not None

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_submit


def _percentile(xs, q):
    return float(np.percentile(np.asarray(xs, dtype=np.float64), q)) if len(xs) else None


class DoseServer:
    """Admission, continuous batching and completion over an executor.

    The executor provides ``n_slots``, ``fixed_bytes()``,
    ``output_bytes(request)``, ``wave_key(request)``, ``scratch_bytes(slot)``,
    ``scratch_growth(slot, items)``, ``scratch_total(items)``,
    ``launch(slot, items)``, ``done(slot)``, ``collect(slot)`` (raises if the
    batch failed), ``release(request)`` and ``trim(slot)``.  ``items`` are
    (request, beam index) pairs.  ``scratch_cap`` defaults to the scratch of
    ``max_wave_beams`` beams of the largest request seen by
    ``executor.default_scratch_cap``.
    """

    def __init__(self, executor, budget_bytes, max_wave_beams=32, scratch_cap=None, clock=time.perf_counter):
        self.ex = executor
        self.budget = int(budget_bytes)
        self.max_wave = int(max_wave_beams)
        self.cap = int(scratch_cap if scratch_cap is not None else executor.default_scratch_cap(max_wave_beams))
        self.clock = clock
        self.queue = deque()          # submitted, waiting for memory
        self.ready = deque()          # admitted beams not yet launched: (request, beam index)
        self.busy = {}                # slot -> items on the GPU
        self.reserved = 0             # output bytes of admitted, undelivered requests
        self.finished = []
        self.peak_used = 0
        self.waves = []               # beams per launched batch

    # ------------------------------------------------------------ client --
    def submit(self, request):
        request.t_submit = self.clock()
        self.queue.append(request)
        return request

    def idle(self):
        return not (self.queue or self.ready or self.busy)

    def used(self):
        """Bytes the budget is charged with: fixed + scratch pools + outputs."""
        return self.ex.fixed_bytes() + self.ex.n_slots * self.cap + self.reserved

    def held(self):
        """Bytes actually held: fixed + scratch arenas + outputs."""
        return (self.ex.fixed_bytes() + sum(self.ex.scratch_bytes(s) for s in range(self.ex.n_slots)) +
                self.reserved)

    # --------------------------------------------------------- scheduling --
    def step(self):
        """One scheduler pass: retire finished batches, admit, launch.
        Returns the requests completed in this pass."""
        done = self._retire()
        self._admit()
        self._launch()
        self.peak_used = max(self.peak_used, self.held())
        return done

    def _retire(self):
        out = []
        for slot in list(self.busy):
            if not self.ex.done(slot):
                continue
            items = self.busy.pop(slot)
            err = None
            try:
                self.ex.collect(slot)
            except Exception as e:          # the whole batch failed (e.g. a parallel ray)
                err = e
            now = self.clock()
            for req, _ in items:
                if err is not None and req.error is None:
                    req.error = err
                req.remaining -= 1
                if req.remaining == 0:
                    req.t_done = now
                    self.ex.release(req)
                    self.reserved -= req.reserved
                    req.reserved = 0
                    out.append(req)
        self.finished.extend(out)
        return out

    def _refuse(self, req, why):
        self.queue.popleft()
        req.error = MemoryError(why)
        req.t_done = self.clock()
        self.finished.append(req)

    def _admit(self):
        while self.queue:
            req = self.queue[0]
            need = self.ex.output_bytes(req)
            one = max(self.ex.scratch_total([(req, b)]) for b in range(len(req.beams)))
            if one > self.cap:
                self._refuse(req, f"one beam needs {one} bytes of scratch; a slot's pool is {self.cap}")
                continue
            if self.used() + need > self.budget:
                if self.busy or self.ready or self.reserved:
                    return                   # wait for outputs to be delivered
                self._refuse(req, f"request needs {need} bytes of outputs; budget {self.budget}, "
                                  f"fixed {self.ex.fixed_bytes()}, scratch pools {self.ex.n_slots * self.cap}")
                continue
            self.queue.popleft()
            req.reserved = need
            self.reserved += need
            req.t_admit = self.clock()
            self.ready.extend((req, b) for b in range(len(req.beams)))

    def _take_wave(self):
        """Oldest ready beams that share the first one's key, up to the cap."""
        key = self.ex.wave_key(self.ready[0][0])
        wave, rest = [], deque()
        while self.ready and len(wave) < self.max_wave:
            item = self.ready.popleft()
            (wave if self.ex.wave_key(item[0]) == key else rest).append(item)
        rest.extend(self.ready)
        self.ready = rest
        return wave

    def _fits(self, slot, wave):
        return self.ex.scratch_bytes(slot) + self.ex.scratch_growth(slot, wave) <= self.cap

    def _launch(self):
        for slot in range(self.ex.n_slots):
            if not self.ready:
                return
            if slot in self.busy:
                continue
            wave = self._take_wave()
            # cut the batch until the slot's arena fits its pool; a single
            # beam fits an emptied arena (checked at admission)
            while len(wave) > 1 and not self._fits(slot, wave):
                self.ready.appendleft(wave.pop())
            if not self._fits(slot, wave):
                self.ex.trim(slot)
            self.ex.launch(slot, wave)
            now = self.clock()
            for req, _ in wave:
                if req.t_launch is None:
                    req.t_launch = now
            self.busy[slot] = wave
            self.waves.append(len(wave))

    def run(self, poll_s=100e-6, timeout_s=600.0):
        """Step until every submitted request is finished."""
        t0 = self.clock()
        while not self.idle():
            if not self.step() and self.busy:
                time.sleep(poll_s)
            if self.clock() - t0 > timeout_s:
                raise TimeoutError("dose server did not drain")
        return self.finished

    # -------------------------------------------------------------- stats --
    def stats(self, requests=None):
        reqs = [r for r in (self.finished if requests is None else requests) if r.error is None and r.done]
        lat = [r.latency * 1e3 for r in reqs]
        beams = sum(len(r.beams) for r in reqs)
        if reqs:
            span = max(r.t_done for r in reqs) - min(r.t_submit for r in reqs)
        else:
            span = 0.0
        # the slowest requests, split into waiting for memory (submit ->
        # admit), waiting for a slot (admit -> first launch) and on the GPU
        # (first launch -> done, the dose copy to the host included)
        slow = sorted(reqs, key=lambda r: r.latency, reverse=True)[:3]
        tail = [{"ms": 1e3 * r.latency, "phantom": r.phantom, "beams": len(r.beams),
                 "admit_ms": 1e3 * (r.t_admit - r.t_submit),
                 "to_launch_ms": 1e3 * (r.t_launch - r.t_admit) if r.t_launch is not None else None,
                 "on_gpu_ms": 1e3 * (r.t_done - r.t_launch) if r.t_launch is not None else None}
                for r in slow]
        return {"requests": len(reqs), "beams": beams,
                "p50_ms": _percentile(lat, 50), "p99_ms": _percentile(lat, 99),
                "beams_per_s": beams / span if span > 0 else None,
                "mean_batch_beams": float(np.mean(self.waves)) if self.waves else None,
                "peak_bytes": self.peak_used, "budget_bytes": self.budget, "slowest": tail}


class GpuExecutor:
    """Slots are dose plans with their own CUDA stream on one device.

    Phantoms are registered once and stay resident (``add_phantom``).  Each
    slot's plan keeps its kernel tables and stencils; ``prepare`` builds the
    stencils for the largest grid up front so no request pays for it.
    """

    def __init__(self, device=0, n_slots=2, copy_to_host=True, tuning=None):
        import torch
        from .engine import DoseEngine
        self.torch = torch
        self.device = torch.device("cuda", int(device))
        self.engines = [DoseEngine(device) for _ in range(n_slots)]
        if tuning:
            for e in self.engines:
                e.set_tuning(**tuning)      # the cone/TERMA schedule (conehead_gb300.autotune)
        self.streams = [torch.cuda.Stream(self.device) for _ in range(n_slots)]
        self.events = [None] * n_slots
        self.batch_log = []
        self.n_slots = n_slots
        self.copy_to_host = copy_to_host
        self.phantoms = {}
        self._phantom_bytes = 0
        self._kernel_keys = {}

    # ------------------------------------------------------- residency --
    def add_phantom(self, name, phantom):
        rho = self.engines[0].upload_densities(phantom.densities)
        self.phantoms[name] = (phantom, rho)
        self._phantom_bytes += rho.numel() * rho.element_size()
        return name

    def prepare(self, settings, spacing, max_size):
        """Kernel tables and stencils for the largest grid, and the stencil
        spectrum of every registered phantom's grid, in every slot."""
        from . import _native as N
        import ctypes
        shapes = [tuple(int(k) for k in max_size)]
        shapes += [tuple(int(k) for k in ph.size) for ph, _ in self.phantoms.values()]
        for eng, st in zip(self.engines, self.streams):
            with self.torch.cuda.stream(st):
                eng.set_kernel(settings["energy_weights"])
                for shape in dict.fromkeys(shapes):
                    g = N.grid_struct(shape, (0.0, 0.0, 0.0), spacing)
                    N.check(eng.L.ch_plan_prepare(eng.plan, ctypes.byref(g), eng.stream()), "ch_plan_prepare")
        self.torch.cuda.synchronize(self.device)

    def warm(self, settings, max_wave_beams, pinned_per_shape=None):
        """Take every first-use cost out of serving: each slot runs one full
        batch of ``max_wave_beams`` beams on the largest registered phantom
        (its scratch arena grows to the pool a server with that batch cap
        charges, so no later batch allocates -- a growth frees the old arena,
        and cudaFree waits for the whole device) and one beam on every other
        phantom (every grid shape's kernels), and the pinned host buffers the
        doses are copied into are allocated once for every phantom shape and
        returned to torch's host cache (a first cudaHostAlloc of tens of MB
        takes milliseconds)."""
        from .block import Block
        from .source import Source
        torch = self.torch
        src = Source()
        src.gantry = 0.0
        src.collimator = 0.0
        blk = Block()
        blk.set_square(5.0)
        names = sorted(self.phantoms, key=lambda k: -int(np.prod(self.phantoms[k][0].size)))
        for slot, eng in enumerate(self.engines):
            with torch.cuda.stream(self.streams[slot]):
                eng.set_kernel(settings["energy_weights"])
                for i, name in enumerate(names):
                    ph, rho = self.phantoms[name]
                    n = max_wave_beams if i == 0 else 1
                    jobs = [eng.job(ph, rho, src, eng.block_for(blk), settings) for _ in range(n)]
                    eng.run_batch(jobs)
                    eng.sync()
        k = pinned_per_shape if pinned_per_shape is not None else self.n_slots * max_wave_beams
        for name in names:
            shape = tuple(int(n) for n in self.phantoms[name][0].size)
            bufs = [torch.empty(shape, dtype=torch.float32, pin_memory=True) for _ in range(k)]
            del bufs
        torch.cuda.synchronize(self.device)

    # ------------------------------------------------------- accounting --
    def _plan_memory(self, eng):
        import ctypes
        from . import _native as N
        tables, scratch = ctypes.c_size_t(), ctypes.c_size_t()
        N.check(eng.L.ch_plan_memory(eng.plan, ctypes.byref(tables), ctypes.byref(scratch)), "ch_plan_memory")
        return tables.value, scratch.value

    def fixed_bytes(self):
        return self._phantom_bytes + sum(self._plan_memory(e)[0] for e in self.engines)

    def scratch_bytes(self, slot):
        return self._plan_memory(self.engines[slot])[1]

    def default_scratch_cap(self, max_wave_beams):
        """Scratch of a full batch of the largest registered phantom."""
        if not self.phantoms:
            return 1 << 30
        big = max(self.phantoms, key=lambda k: int(np.prod(self.phantoms[k][0].size)))
        probe = types.SimpleNamespace(phantom=big)
        return self._scratch(0, [(probe, 0)] * max_wave_beams)[1]

    def output_bytes(self, req):
        ph = self.phantoms[req.phantom][0]
        return 4 * int(np.prod(ph.size)) * len(req.beams)

    def wave_key(self, req):
        ph = self.phantoms[req.phantom][0]
        ew = req.settings["energy_weights"]
        return (tuple(float(np.float32(s)) for s in ph.spacing),
                tuple((k, float(v)) for k, v in ew.items()))

    def _scratch(self, slot, items):
        import ctypes
        from . import _native as N
        eng = self.engines[slot]
        grids = [N.grid_struct(self.phantoms[r.phantom][0].size, self.phantoms[r.phantom][0].origin,
                               self.phantoms[r.phantom][0].spacing) for r, _ in items]
        arr = (N.Grid * len(grids))(*grids)
        growth, total = ctypes.c_size_t(), ctypes.c_size_t()
        N.check(eng.L.ch_batch_scratch_bytes(eng.plan, len(grids), arr, ctypes.byref(growth), ctypes.byref(total)),
                "ch_batch_scratch_bytes")
        return growth.value, total.value

    def scratch_growth(self, slot, items):
        return self._scratch(slot, items)[0]

    def scratch_total(self, items):
        return self._scratch(0, items)[1]

    # -------------------------------------------------------- execution --
    def launch(self, slot, items):
        torch = self.torch
        eng, st = self.engines[slot], self.streams[slot]
        t0 = time.perf_counter()
        with torch.cuda.stream(st):
            e0 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            eng.set_kernel(items[0][0].settings["energy_weights"])
            jobs = []
            for req, b in items:
                ph, rho = self.phantoms[req.phantom]
                src, blk = req.beams[b]
                dose = torch.empty(tuple(int(n) for n in ph.size), dtype=torch.float32, device=self.device)
                jobs.append(eng.job(ph, rho, src, eng.block_for(blk), req.settings, dose=dose))
            eng.run_batch(jobs)
            e1 = torch.cuda.Event(enable_timing=True)
            e1.record(st)
            for (req, b), job in zip(items, jobs):
                if self.copy_to_host:
                    host = torch.empty(job.dose.shape, dtype=torch.float32, pin_memory=True)
                    host.copy_(job.dose, non_blocking=True)
                    req.doses[b] = host
                else:
                    req.doses[b] = job.dose
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(st)
        self.events[slot] = (ev, jobs, e0, e1, time.perf_counter() - t0,
                             sorted({self.phantoms[r.phantom][0].size[0] for r, _ in items}), len(items))

    def done(self, slot):
        ev = self.events[slot]
        return ev is None or ev[0].query()

    def collect(self, slot):
        eng = self.engines[slot]
        ev, _, e0, e1, host_s, sizes, n = self.events[slot]
        # per batch: host time of the launch call, device time of the dose
        # calculation and of the copies to the host (stream-ordered events, so
        # the time includes waiting for the other slot's work on the GPU)
        self.batch_log.append({"slot": slot, "beams": n, "grids": sizes, "host_ms": 1e3 * host_s,
                               "device_ms": e0.elapsed_time(e1), "copy_ms": e1.elapsed_time(ev)})
        self.events[slot] = None
        with self.torch.cuda.stream(self.streams[slot]):
            eng.sync()                      # the stream is idle: reads the device error flags

    def release(self, req):
        pass                                # device outputs go back to torch's cache with the jobs

    def trim(self, slot):
        from . import _native as N
        eng = self.engines[slot]
        N.check(eng.L.ch_plan_trim(eng.plan), "ch_plan_trim")

    def close(self):
        for e in self.engines:
            e.close()


def poisson_workload(rng, phantom_names, rate, n_requests, beams_per_request=(1, 8), field=5.0):
    """Arrival times (s) and requests: beams as in the 128^3 workload
    (5 x 5 cm jaws, gantry uniform in [0, 360)), phantoms drawn uniformly."""
    from .phantoms import random_beam
    gaps = rng.exponential(1.0 / rate, n_requests)
    arrivals = np.cumsum(gaps) - gaps[0]
    specs = []
    for _ in range(n_requests):
        name = phantom_names[int(rng.integers(0, len(phantom_names)))]
        nb = int(rng.integers(beams_per_request[0], beams_per_request[1] + 1))
        specs.append((name, [random_beam(rng, field=field) for _ in range(nb)]))
    return arrivals, specs


def drive(server, arrivals, specs, settings, poll_s=50e-6, timeout_s=600.0, on_done=None):
    """Submit requests at their arrival times (open loop) and step the server
    until all are done; returns the requests in submission order.
    ``on_done(request)`` is called as each one finishes (e.g. to drop its
    dose arrays)."""
    clock = server.clock
    t0 = clock()
    reqs = []
    i = 0
    while i < len(arrivals) or not server.idle():
        now = clock() - t0
        while i < len(arrivals) and arrivals[i] <= now:
            name, beams = specs[i]
            reqs.append(server.submit(Request(name, beams, settings)))
            i += 1
        progressed = server.step()
        if on_done is not None:
            for r in progressed:
                on_done(r)
        if not progressed:
            wait = poll_s
            if i < len(arrivals):
                wait = min(wait, max(0.0, arrivals[i] - (clock() - t0)))
            if wait > 0:
                time.sleep(wait)
        if clock() - t0 > timeout_s:
            raise TimeoutError("workload did not finish")
    return reqs
