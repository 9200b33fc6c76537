"""Benchmark: beams/s of the collapsed-cone dose engine on GB300.

Workload (one "step"): a batch of --beams beams (default 32: one cull, one
TERMA and one spectral launch of 16 beam pairs) on the heterogeneous 128^3
slab phantom (0.25 cm voxels: water, lung slab 0.25 g/cc at depth 5-12 cm,
bone slab 1.85 g/cc at 14-16 cm, 20 random cuboid inserts of 0.2-2.0
g/cc), 5 x 5 cm^2 jaw field, gantry uniform in [0, 360), seeded synthetic
inputs.  Every beam runs the whole path: blocking -> radiological depth ->
fluence -> TERMA -> collapsed-cone dose (float32 dose and accumulation).

  value       beams/s with inputs resident in HBM (one batched call per
              step; the host enqueues step s + 1 while the device runs step
              s), L2 flushed (256 MiB write) between steps, outside the
              per-step event windows
  e2e         beams/s through the C ABI with pinned host buffers: density
              (and any block map that exists; a jaw field travels as its
              rectangle in the beam record) H2D plus dose D2H inside the
              timed region
  roofline    the cone stage of the schedule in use, from the library's stage
              events on the launching stream, against the measured HBM peak:
              achieved = the stage's algorithmic bytes, 8 N per beam (TERMA
              read, dose write), over its time; traffic = the DRAM bytes of
              the committed ncu capture, and their ratio to the algorithmic
              bytes; pass_traffic_frac (spectral) = the bytes the five FFT
              passes' structure must move (A and B intermediates written and
              read twice, S^ once per launch) over the same time.  "onchip"
              (gather) gives its updates/s against the shared-memory lane
              ceiling; "updates" gives the reference-equivalent updates/s of
              the cone stage against an FP32 FMA ceiling
  cpu_baseline / --impl reference
              the CPU oracle (C++ FP64 restatement of the reference path,
              OpenMP over every host core) on whole beams of the workload
  batched_captured
              64 beams on mixed 64^3-160^3 slab phantoms (jaws U[2,20] cm,
              gantry U[0,360), collimator U[0,90)) in one captured CUDA graph
              with the autotuned schedule
  adjoint     forward dose and beamlet-weight gradient (ch_dose_adjoint) on
              the 128^3 phantom with 40 x 40 beamlets of 0.5 cm
  serving     the continuous-batching server (conehead_gb300.serving) under
              open-loop Poisson arrivals: requests of 1-8 beams (5 x 5 cm,
              gantry U[0, 360)) on resident slab phantoms of 64^3, 96^3,
              128^3 and 192^3, HBM budget 80% of the device, doses copied to
              pinned host memory; p50/p99 request latency and beams/s per rate

Multi-GPU (torchrun): beams are independent, so each rank runs its own
batches (weak scaling, no data-path collective); the step time is the
maximum over ranks.
"""
import argparse
import contextlib
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

METRIC = ("beams/s @128³ batched vs plain-GPU vs CPU at ≤0.5% Dmax; HBM GB/s; "
          "p50/p99 ms")
SETTINGS = {
    'sPri': 0.90924, 'sAnn': 2.887e-3, 'zAnn': 4.0, 'rInner': 0.2, 'rOuter': 1.4,
    'zExp': 12.5, 'sExp': 8.289e-3, 'kExp': 0.4816, 'softRatio': 0.0025,
    'softLimit': 20, 'hornRatio': 0.0065, 'fluenceResampling': 3,
    'energy_weights': {"0.5": 0.08196, "1.0": 0.12385, "1.5": 0.10605, "2.0": 0.08307,
                       "2.5": 0.05881, "3.0": 0.03911, "3.5": 0.02131, "4.0": 0.02426,
                       "4.5": 0.0, "5.0": 0.00881, "5.5": 0.0, "6.0": 0.00498},
}


def host_link_rate(dev_bufs, host_bufs, stream, reps=3):
    """GB/s of the machine's host link on the e2e loop's own buffers (one step's
    doses and their pinned host copies), measured after the timed region:
    device -> host and host -> device, one copy per buffer, CUDA events on
    the copy stream."""
    import torch
    nbytes = sum(t.numel() * t.element_size() for t in dev_bufs)
    out = {}
    for name, pairs in (("d2h_gbs", list(zip(host_bufs, dev_bufs))), ("h2d_gbs", list(zip(dev_bufs, host_bufs)))):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(reps):
                for dst, src in pairs:
                    dst.copy_(src, non_blocking=True)
            e1.record(stream)
        e1.synchronize()
        out[name] = reps * nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9
    out["bytes"] = nbytes
    return out


@contextlib.contextmanager
def quiet_gc():
    """Collect once, then keep Python's cyclic collector out of a timed loop
    whose window includes the host enqueueing the steps: a pass over this
    process's objects can stall that thread for tens of milliseconds."""
    gc.collect()
    gc.freeze()
    gc.disable()
    try:
        yield
    finally:
        gc.enable()
        gc.unfreeze()


# ----------------------------------------------------------- distribution --

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_init(backend):
    import torch.distributed as dist
    world, rank, _ = dist_env()
    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend, rank=rank, world_size=world)
    return world, rank


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(x, device=None):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def beam_seed(rank, index):
    """Per-rank, per-beam seed: ranks draw disjoint beams (weak scaling)."""
    return 1_000_003 * (rank + 1) + index


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    """nvidia-smi samples (every 20 ms) of the SM clock, its maximum, power and
    the throttle reasons.  Started before the timed loops and waited on until
    its first sample arrives (nvidia-smi takes a while to start); the timed
    loops mark their windows with begin() / end(), and stop() summarises the
    samples that arrived inside a window."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []      # (arrival time, fields)
        self.windows = []
        self.proc = None
        self.thread = None
        self.first = threading.Event()

    def start(self, wait_s=5.0):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        self.first.wait(wait_s)

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.monotonic(), [p.strip() for p in line.split(",")]))
            self.first.set()

    def begin(self):
        self.windows.append([time.monotonic(), None])

    def end(self):
        if self.windows and self.windows[-1][1] is None:
            self.windows[-1][1] = time.monotonic()

    def stop(self):
        if self.proc is None:
            return self.summary()
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        return self.summary()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        samples = list(self.samples)
        inside = [f for t, f in samples
                  if any(a <= t <= (b if b is not None else float("inf")) for a, b in self.windows)]
        rows = inside or [f for _, f in samples]
        sm = [float(r[0]) for r in rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if len(r) > 3 + i and r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside),
                "windows_ms": [round((b - a) * 1e3, 1) for a, b in self.windows if b is not None],
                "basis": "samples inside the timed windows (device-timed loop and e2e loop)"
                         if inside else "no sample inside the timed windows: every sample of the run"}


# --------------------------------------------------------------- workload --
def host_cpu():
    """The host CPU model (lscpu, else /proc/cpuinfo) and its online cores."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if model is None:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    import platform
    return {"model": model, "machine": platform.machine(), "online_cores": os.cpu_count()}


def workload(n, spacing, seed=0):
    from conehead_gb300.phantoms import slab_phantom
    return slab_phantom(n, spacing, seed=seed)


def make_beam(seed, field):
    from conehead_gb300.phantoms import random_beam
    return random_beam(np.random.default_rng(seed), field=field)


def cpu_oracle_beams(phantom, beams, threads=None):
    """Time the FP64 oracle on whole beams; returns (beams/s, cores, seconds)."""
    from oracle import oracle
    oracle.build()
    t0 = time.perf_counter()
    for src, blk in beams:
        oracle.calculate(src, blk, phantom, SETTINGS, oracle.MODE_F64)
    dt = time.perf_counter() - t0
    return len(beams) / dt, oracle.num_threads(), dt


def run_reference(args):
    """--impl reference: the CPU oracle of the reference path, rank 0 only."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    ph = workload(args.grid, args.spacing)
    beams = [make_beam(beam_seed(0, i), args.field) for i in range(args.warmup + args.steps)]
    from oracle import oracle
    oracle.build()
    for src, blk in beams[:args.warmup]:
        oracle.calculate(src, blk, ph, SETTINGS, oracle.MODE_F64)
    v, cores, dt = cpu_oracle_beams(ph, beams[args.warmup:])
    sample = (f"{args.steps} whole beams ({args.grid}^3, {args.field:g}x{args.field:g} cm, "
              f"random gantry), one per step: a bounded sample of the {args.beams}-beam step; FP64 oracle, "
              f"OpenMP")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "beams/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config(args),
        "cpu_baseline": {"value": v, "unit": "beams/s", "cores": cores, "kind": "port", "sample": sample,
                         "cpu": host_cpu()},
        "e2e": {"value": v, "unit": "beams/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))
    return 0


def serving_extras(args, dev):
    """Poisson-arrival serving runs, one per rate; results dropped as they land."""
    import torch
    from conehead_gb300.serving import DoseServer, GpuExecutor, drive, poisson_workload
    from conehead_gb300.conehead import engine
    sizes = (64, 96, 128, 192)
    # the schedule the headline run tuned (the default if it did not tune)
    ex = GpuExecutor(dev.index, n_slots=2, tuning=engine(dev.index).get_tuning())
    for n in sizes:
        ex.add_phantom(f"p{n}", workload(n, args.spacing, seed=n))
    ex.prepare(SETTINGS, (args.spacing,) * 3, (max(sizes),) * 3)
    # every slot's arena at its full pool, every shape's kernels and pinned
    # host buffers allocated: no request pays a first-use cost
    if not args.serve_no_warm:
        ex.warm(SETTINGS, args.serve_batch)
    budget = int(0.8 * torch.cuda.mem_get_info(dev)[1])
    names = [f"p{n}" for n in sizes]

    def drop(req):
        assert req.error is None, req.error
        req.doses = None

    # warm-up (pinned host buffers, lazy CUDA state), not reported
    arr, specs = poisson_workload(np.random.default_rng(99), names, 400.0, 24)
    drive(DoseServer(ex, budget, max_wave_beams=args.serve_batch), arr, specs, SETTINGS, on_done=drop)
    # a long-running server collects once after start-up and freezes what it
    # holds: otherwise a cyclic-GC pass over the objects of this process
    # (every earlier section's beams and jobs) stalls the scheduler loop for
    # tens of milliseconds in the middle of the timed rates
    gc.collect()
    gc.freeze()
    rows = []
    for rate in args.serve_rates:
        rng = np.random.default_rng(int(rate))
        arr, specs = poisson_workload(rng, names, float(rate), args.serve_requests)
        server = DoseServer(ex, budget, max_wave_beams=args.serve_batch)
        ex.batch_log.clear()
        drive(server, arr, specs, SETTINGS, on_done=drop)
        st = server.stats()
        blog = ex.batch_log
        batches = {"n": len(blog),
                   "host_ms_median": statistics.median(b["host_ms"] for b in blog) if blog else None,
                   "device_ms_median": statistics.median(b["device_ms"] for b in blog) if blog else None,
                   "copy_ms_median": statistics.median(b["copy_ms"] for b in blog) if blog else None,
                   "slowest": sorted(blog, key=lambda b: -(b["device_ms"] + b["copy_ms"]))[:3]}
        rows.append({"rate_req_s": rate, "requests": st["requests"], "beams": st["beams"],
                     "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "beams_per_s": st["beams_per_s"],
                     "mean_batch_beams": st["mean_batch_beams"], "peak_gb": st["peak_bytes"] / 1e9,
                     "slowest": st["slowest"], "batches": batches})
    ex.close()
    gc.unfreeze()
    return {"workload": "Poisson arrivals, 1-8 beams per request (5x5 cm, gantry U[0,360)), phantoms "
                        "64^3/96^3/128^3/192^3 @ 0.25 cm resident, 2 slots, latency = arrival to dose "
                        "in pinned host memory",
            "budget_gb": budget / 1e9, "max_batch_beams": args.serve_batch, "rates": rows}


def adjoint_extras(args, dev):
    """Beamlet-weight gradient at 128^3: 40 x 40 beamlets of 0.5 cm, weights
    U[0, 1], L = sum (dose - target)^2 with target 2 in a 2 cm-radius sphere.
    Times (CUDA events on the engine's stream) the forward dose, the objective
    gradient in torch, and ch_dose_adjoint."""
    import torch
    from conehead_gb300.adjoint import BeamletDose, BeamletGrid, sphere_target
    from conehead_gb300.conehead import engine
    from conehead_gb300 import Source
    rng = np.random.default_rng(7)
    ph = workload(args.grid, args.spacing)
    target = torch.from_numpy(sphere_target(ph, tuple(rng.uniform(-3, 3, 3)), 2.0)).to(dev)
    src = Source()
    src.gantry = float(rng.uniform(0, 360))
    src.collimator = 0.0
    bl = BeamletGrid.square(40, 0.5)
    op = BeamletDose(engine(dev.index), ph, src, bl, SETTINGS)
    w = torch.tensor(rng.uniform(0, 1, bl.shape).astype(np.float32), device=dev)
    st = torch.cuda.current_stream(dev)
    fwd, bwd = [], []
    for it in range(args.adjoint_iters + 3):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(st)
        dose = op.forward(w)
        e1.record(st)
        grad_dose = 2.0 * (dose - target)
        g = op.backward(grad_dose)
        e2.record(st)
        e2.synchronize()
        if it >= 3:
            fwd.append(e0.elapsed_time(e1))
            bwd.append(e1.elapsed_time(e2))
    op.eng.sync()
    assert float(g.abs().max()) > 0
    return {"workload": f"{args.grid}^3 slab phantom @ {args.spacing:g} cm, 40x40 beamlets of 0.5 cm, "
                        "weights U[0,1], L = sum (dose - target)^2",
            "forward_ms": statistics.median(fwd), "gradient_ms": statistics.median(bwd),
            "gradient_evals_per_s": 1000.0 / (statistics.median(fwd) + statistics.median(bwd)),
            "iters": len(fwd)}


def batched_extras(args, dev):
    """64 beams in one captured launch: heterogeneous slab phantoms of 64^3,
    96^3, 128^3 and 160^3 at 0.25 cm, jaws X and Y each U[2, 20] cm, gantry
    U[0, 360), collimator U[0, 90); schedule from the autotuner.  Times graph
    replays (CUDA events, L2 flushed between replays) and, for reference, the
    same batch uncaptured with the default schedule."""
    import torch
    from conehead_gb300.autotune import autotune, time_batch
    from conehead_gb300.engine import DoseEngine
    from conehead_gb300.phantoms import random_beam
    eng = DoseEngine(dev.index)
    eng.set_kernel(SETTINGS["energy_weights"])
    sizes = (64, 96, 128, 160)
    phantoms = {n: workload(n, args.spacing, seed=n) for n in sizes}
    rhos = {n: eng.upload_densities(ph.densities) for n, ph in phantoms.items()}
    rng = np.random.default_rng(64)
    jobs, grid_of = [], []
    for i in range(args.batch_beams):
        n = sizes[int(rng.integers(0, len(sizes)))]
        src, blk = random_beam(rng, rect=(2.0, 20.0), collimator=True)
        jobs.append(eng.job(phantoms[n], rhos[n], src, eng.block_for(blk), SETTINGS))
        grid_of.append(n)
    eng.prepare((max(sizes),) * 3, (args.spacing,) * 3)
    eng.set_tuning()
    default_ms = time_batch(eng, jobs, iters=2)
    tuned = autotune(eng, jobs)
    batch = eng.capture(jobs)
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    ms = []
    for it in range(args.batch_iters + 2):
        flush.fill_(float(it))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        batch.launch()
        e1.record(st)
        e1.synchronize()
        if it >= 2:
            ms.append(e0.elapsed_time(e1))
    batch.sync()
    batch.close()
    eng.close()
    med = statistics.median(ms)
    # kernels in the graph: scratch reset, cull, TERMA, then per grid shape
    # its spectral launches (three kernels on the plane path, five on the
    # five-pass one), or the tap ranges and the gather
    if int(tuned["tuning"].get("cone_method", 0)) == 0:
        per_shape = {n: grid_of.count(n) for n in set(grid_of)}
        kernels = 3 + sum(spectral_launches(k) * (3 if plane_path((n, n, n)) else 5) for n, k in per_shape.items())
    else:
        kernels = 5
    return {"workload": f"{args.batch_beams} beams, slab phantoms 64^3/96^3/128^3/160^3 @ {args.spacing:g} cm, "
                        "jaws U[2,20] cm, gantry U[0,360), collimator U[0,90), one captured CUDA graph",
            "beams_per_s": args.batch_beams * 1000.0 / med, "ms_per_batch": med,
            "uncaptured_default_schedule_ms": default_ms, "tuning": tuned["tuning"],
            "tuned_uncaptured_ms": tuned["ms"], "autotune_cached": tuned["cached"],
            "kernels_per_batch": kernels, "graph_launches_per_batch": 1}


def reference_updates(eng, ph, jobs):
    """Voxel·direction updates the reference's cone scatter does per beam
    (conehead/conehead.py:385-488): for every voxel with TERMA != 0, each of
    the 576 directions (the 12 phi = 180 deg repeats included), one update per
    voxel its DDA walk visits inside the grid.  Walk offsets come from the
    library's DDA hook traced from the centre of a (2n - 1) grid (every offset
    two voxels of the n grid can have), the TERMA support from the beam's
    intermediates; counted with a summed-area table.  Mean over `jobs`."""
    from conehead_gb300.engine import dda_trace
    n = [int(k) for k in ph.size]
    dirs = eng.cone_directions()
    big = [2 * k - 1 for k in n]
    c = np.array([k - 1 for k in n], dtype=np.int32)
    vox, _, ln = dda_trace(big, [float(x) for x in ph.spacing], np.tile(c, (len(dirs), 1)), dirs,
                           cap=sum(big) + 2, device=eng.device.index)
    offs = [vox[u, :ln[u]] - c for u in range(len(dirs))]
    per_beam = []
    for job in jobs:
        _, inter = eng.run(job, intermediates=True)
        eng.sync()
        mask = (inter["terma"] != 0).cpu().numpy()
        S = np.zeros([k + 1 for k in n], dtype=np.int64)
        S[1:, 1:, 1:] = mask.astype(np.int64).cumsum(0).cumsum(1).cumsum(2)
        total = 0
        for O in offs:
            lo = np.clip(-O, 0, None)                          # sources s with s + O inside the grid
            hi = np.minimum(np.array(n) - 1 - O, np.array(n) - 1) + 1
            ok = np.all(hi > lo, axis=1)
            lo, hi = lo[ok], hi[ok]
            x0, y0, z0 = lo.T
            x1, y1, z1 = hi.T
            total += int((S[x1, y1, z1] - S[x0, y1, z1] - S[x1, y0, z1] - S[x1, y1, z0] + S[x0, y0, z1]
                          + S[x0, y1, z0] + S[x1, y0, z0] - S[x0, y0, z0]).sum())
        per_beam.append(total)
    return float(np.mean(per_beam))


def stage_rooflines(stats, beams, n_vox, cone_bytes, cone_ms, hbm_peak, method):
    """Each stage's achieved HBM rate on its algorithmic bytes (CUDA events
    the library records on the launching stream), against the measured peak.
    prologue: the density read and the TERMA write, 8 N bytes per beam (the
    per-ray density gathers hit L2); cone: as in `roofline`."""
    pro_ms = statistics.mean(x["ms_prologue"] for x in stats)
    pro_bytes = beams * 8 * n_vox
    out = {"prologue": {"ms": pro_ms, "algorithmic_bytes": pro_bytes,
                        "achieved_gbs": pro_bytes / (pro_ms * 1e-3) / 1e9,
                        "frac": pro_bytes / (pro_ms * 1e-3) / 1e9 / hbm_peak,
                        "bound": "instruction issue (exact DDA per listed voxel)"},
           "cone": {"ms": cone_ms, "algorithmic_bytes": cone_bytes,
                    "achieved_gbs": cone_bytes / (cone_ms * 1e-3) / 1e9,
                    "frac": cone_bytes / (cone_ms * 1e-3) / 1e9 / hbm_peak,
                    "method": method}}
    return out


def spectral_period(n):
    """FFT period of one axis: the smallest 2^a or 3 * 2^a (a >= 4) >= 2 n - 1."""
    periods = sorted({16 << a for a in range(9)} | {48 << a for a in range(7)})
    return next(m for m in periods if m >= 2 * n - 1)


# beam pairs per spectral launch (SPEC_MAX_PAIRS of the library)
SPEC_MAX_PAIRS = 16


def spectral_launches(beams, max_pairs=SPEC_MAX_PAIRS):
    return ((beams + 1) // 2 + max_pairs - 1) // max_pairs


def plane_path(size):
    """The library's plane path: FFT periods of 256 on every axis (grids of
    97-128 voxels per axis): z forward, one fused plane kernel (y and x
    transforms, the S^ product and their inverses on chip), z inverse."""
    return all(spectral_period(int(k)) == 256 for k in size)


def spectral_bytes(size, beams, max_pairs=SPEC_MAX_PAIRS):
    """HBM bytes the FFT passes must move for `beams` beams of one grid: per
    pair of beams the two TERMA volumes in and two doses out (16 N), the
    intermediate A [nx][ny][Mz] (complex float32) written and read twice,
    B [nx][My][Mz] likewise on the five-pass path (the plane path keeps it on
    chip), and S^ [Mx][My][Mz] read once per launch."""
    nx, ny, nz = (int(k) for k in size)
    Mx, My, Mz = (spectral_period(k) for k in (nx, ny, nz))
    pairs = (beams + 1) // 2
    a = nx * ny * Mz * 8
    b = 0 if plane_path(size) else nx * My * Mz * 8
    return pairs * (16 * nx * ny * nz + 4 * a + 4 * b) + spectral_launches(beams, max_pairs) * Mx * My * Mz * 8


def config(args, beams_per_step=None):
    return {"workload": f"heterogeneous slab phantom {args.grid}^3 @ {args.spacing:g} cm, "
                        f"{args.field:g}x{args.field:g} cm2 field, gantry U[0,360), 6 MV, 12x48 cones",
            "grid": args.grid, "spacing_cm": args.spacing, "field_cm": args.field,
            "beams_per_step": beams_per_step if beams_per_step is not None else args.beams,
            "l2": "flushed between timed steps (256 MiB write)", "seed": 0}


def percentile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = (len(xs) - 1) * q
    lo, hi = int(np.floor(k)), int(np.ceil(k))
    return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)


def run_ours(args):
    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist_init("nccl")
    from conehead_gb300.conehead import engine
    eng = engine(local)
    eng.set_kernel(SETTINGS["energy_weights"])
    ph = workload(args.grid, args.spacing)
    N = int(np.prod(ph.size))
    rho = eng.upload_densities(ph.densities)
    B = args.beams
    total = (args.warmup + args.steps) * B
    beams = [make_beam(beam_seed(rank, i), args.field) for i in range(total)]
    # each beam's block through the public path: a jaw rectangle goes to the
    # device as a rectangle (no map), anything else as its cropped map
    dblocks = [eng.block_for(blk) for _, blk in beams]
    doses = [torch.empty(ph.size, dtype=torch.float32, device=dev) for _ in range(B)]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)

    def step_jobs(s):
        return [eng.job(ph, rho, beams[s * B + i][0], dblocks[s * B + i], SETTINGS, dose=doses[i])
                for i in range(B)]

    # ---- device-resident batched steps
    for s in range(args.warmup):
        eng.run_batch(step_jobs(s))
    eng.sync()
    # schedule for this workload from the autotuner (untimed, cached per device and workload)
    schedule = {"tuning": eng.get_tuning(), "source": "default"}
    if not args.no_autotune:
        from conehead_gb300.autotune import autotune
        r = autotune(eng, step_jobs(0))
        schedule = {"tuning": r["tuning"], "source": "autotune (cached)" if r["cached"] else "autotune"}
    # The host enqueues step s + 1 (building its jobs and launch records)
    # while the device runs step s, as a batch loop does; each step's window
    # runs from after its L2 flush to the end of its batch, so the flushes are
    # outside and no host preparation leaves the device idle inside.
    # (job descriptors are host objects, built before the timed loop as the
    # e2e loop builds its sets' once; each call still stages its own launch
    # records)
    timed_jobs = {s: step_jobs(s) for s in range(args.warmup, args.warmup + args.steps)}
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    marks = []
    with quiet_gc():
        clocks.begin()
        for s in range(args.warmup, args.warmup + args.steps):
            jobs = timed_jobs[s]
            flush.fill_(float(s))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            eng.run_batch(jobs)
            e1.record(st)
            marks.append((e0, e1))
        torch.cuda.synchronize(dev)
        clocks.end()
    barrier()
    eng.sync()
    step_ms = [a.elapsed_time(b) for a, b in marks]
    # Stage times (prologue, cone stage) from the library's events, which
    # hold one call's: the timed steps replayed one at a time after the timed
    # loop, same jobs and flushes, each call's events read before the next.
    stats = []
    for s in range(args.warmup, args.warmup + args.steps):
        flush.fill_(float(s))
        eng.run_batch(timed_jobs[s])
        eng.sync()
        stats.append(eng.stats())
    local_s = sum(step_ms) / 1000.0
    job_s = max_over_ranks(local_s, dev)
    value = world * args.steps * B / job_s

    # ---- cone stage roofline (the library's stage events, same stream)
    cone_ms = statistics.mean(x["ms_cone"] for x in stats)
    updates = statistics.mean(x["updates"] for x in stats)
    method = "spectral" if int(eng.get_tuning().get("cone_method", 0)) == 0 else "gather"
    # algorithmic bytes of the cone stage: TERMA read + dose write, 8 N per
    # beam, whatever the method (the per-beam figure of the path's roofline)
    alg_bytes = B * 2 * 4 * N
    if method == "spectral":
        pass_bytes = spectral_bytes(ph.size, B)
        # scratch reset, cull, TERMA (every beam in one launch each), then
        # per spectral launch three kernels (plane path: z forward, plane
        # kernel, z inverse) or five passes
        launches_per_step = 3 + (3 if plane_path(ph.size) else 5) * spectral_launches(B)
    else:
        pass_bytes = alg_bytes
        launches_per_step = 5                     # reset, cull, TERMA, tap ranges, gather
    peaks = {}
    pk_path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / (cone_ms * 1e-3) / 1e9
    # DRAM bytes of one cone launch: the ncu capture's bytes per beam (it reads
    # each beam's TERMA once) times the beams of this launch
    traffic = None
    tr_path = os.path.join(HERE, "profiles", f"{'spectral' if method == 'spectral' else 'cone_gather'}"
                                             f"_128cube_dram.json")
    if os.path.exists(tr_path) and args.grid == 128:
        with open(tr_path) as f:
            tr = json.load(f)
        if tr.get("dram_bytes_per_beam"):
            traffic = tr["dram_bytes_per_beam"] * B
    props = torch.cuda.get_device_properties(dev)
    sm_mhz = clocks.summary().get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    onchip = None
    if method == "gather":
        lds_ceiling = props.multi_processor_count * 32 * sm_mhz * 1e6     # one 4-byte LDS lane per update
        onchip = {"metric": "voxel-direction updates/s", "achieved": updates / (cone_ms * 1e-3),
                  "peak": lds_ceiling, "frac": updates / (cone_ms * 1e-3) / lds_ceiling,
                  "peak_basis": "SMs x 32 shared-memory lanes/clk x median SM clock"}
    # a direct sum of the reference's updates costs one FP32 FMA each
    fma_ceiling = props.multi_processor_count * 128 * sm_mhz * 1e6

    # ---- e2e through the C ABI with pinned host buffers.  Every step copies
    # its density and block crops host -> device, runs the batch and copies
    # every dose device -> host.  Two buffer sets and three streams pipeline
    # the steps: step s + 1's inputs go up (copy-in stream) and step s - 1's
    # doses come down (copy-out stream) while step s computes.  The timed
    # region runs from the first copy in to the last copy out, the L2 flush
    # of each step included.
    # every rank runs it (the window is a max over ranks)
    from conehead_gb300.engine import DeviceBlock
    h_rho = torch.from_numpy(np.ascontiguousarray(ph.densities)).pin_memory()
    # block maps that exist (MLC or drawn maps) are inputs copied every
    # step; a jaw rectangle travels in the beam record
    crops = [i for i in range(B) if dblocks[i].crop is not None]
    h_blocks = {i: torch.from_numpy(np.ascontiguousarray(dblocks[i].crop.cpu().numpy())).pin_memory()
                for i in crops}
    sets = 2
    h_doses = [[torch.empty(ph.size, dtype=torch.float32).pin_memory() for _ in range(B)] for _ in range(sets)]
    d_rho = [torch.empty_like(rho) for _ in range(sets)]
    d_blocks = [{i: torch.empty_like(dblocks[i].crop) for i in crops} for _ in range(sets)]
    d_doses = [[torch.empty(ph.size, dtype=torch.float32, device=dev) for _ in range(B)] for _ in range(sets)]
    in_st, out_st = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    computed, uploaded, copied = [None] * sets, [None] * sets, [None] * sets
    # the job descriptors of a buffer set point at its device buffers and
    # do not change between steps (the data they point at does): built once
    set_jobs = [[eng.job(ph, d_rho[k], beams[i][0],
                         DeviceBlock(d_blocks[k][i], dblocks[i].r0, dblocks[i].c0, dblocks[i].full_shape,
                                     dblocks[i].uniform) if i in d_blocks[k] else dblocks[i],
                         SETTINGS, dose=d_doses[k][i]) for i in range(B)] for k in range(sets)]

    def upload(s):
        k = s % sets
        if computed[k] is not None:
            in_st.wait_event(computed[k])     # step s - 2 no longer reads set k's inputs
        with torch.cuda.stream(in_st):
            d_rho[k].copy_(h_rho, non_blocking=True)
            for i in crops:
                d_blocks[k][i].copy_(h_blocks[i], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(in_st)
        uploaded[k] = ev

    def compute(s):
        k = s % sets
        flush.fill_(float(s))
        st.wait_event(uploaded[k])
        if copied[k] is not None:
            st.wait_event(copied[k])          # set k's doses of step s - 2 are on the host
        eng.run_batch(set_jobs[k])
        done = torch.cuda.Event()
        done.record(st)
        computed[k] = done
        out_st.wait_event(done)
        with torch.cuda.stream(out_st):
            for i in range(B):
                h_doses[k][i].copy_(d_doses[k][i], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(out_st)
        copied[k] = ev

    def run_steps(first, count):
        upload(first)
        for s in range(first, first + count):
            if s + 1 < first + count:
                upload(s + 1)
            compute(s)

    run_steps(0, args.warmup)
    torch.cuda.synchronize(dev)
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # the window spans host enqueueing: the cyclic collector stays out of it
    with quiet_gc():
        clocks.begin()
        # e0 is recorded on the compute stream before the first upload is issued
        e0.record(st)
        in_st.wait_event(e0)
        run_steps(args.warmup, args.steps)
        for ev in copied:
            if ev is not None:
                st.wait_event(ev)
        e1.record(st)
        e1.synchronize()
        clocks.end()
    clk = clocks.stop()
    eng.sync()
    e2e_s = max_over_ranks(e0.elapsed_time(e1) / 1000.0, dev)
    h2d = h_rho.numel() * 4 + sum(h.numel() * 4 for h in h_blocks.values())
    e2e = {"value": world * args.steps * B / e2e_s, "unit": "beams/s",
           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(B * N * 4),
           "pipelined": "two buffer sets, copy-in / compute / copy-out streams: step s+1's inputs and "
                        "step s-1's doses move while step s computes; each set's job descriptors built once",
           "host_link": host_link_rate(d_doses[0], h_doses[0], out_st)}

    # ---- reference-equivalent voxel·direction updates/s (untimed, a few beams)
    updates_line = None
    if rank == 0 and args.update_beams > 0:
        w = reference_updates(eng, ph, [eng.job(ph, rho, beams[i][0], dblocks[i], SETTINGS)
                                        for i in range(min(args.update_beams, B))])
        cone_rate = w * B / (cone_ms * 1e-3)
        updates_line = {"metric": "reference-equivalent voxel·direction updates/s", "per_beam": w,
                        "value": w * value, "e2e_value": w * e2e["value"] if e2e else None,
                        "cone_stage_value": cone_rate,
                        "fp32_fma_ceiling": fma_ceiling,
                        "frac_of_fma_ceiling": cone_rate / fma_ceiling,
                        "ceiling_basis": "a direct sum costs one FP32 FMA per update: SMs x 128 lanes x "
                                         "median SM clock",
                        "basis": "updates the reference's per-voxel cone scatter does per beam (every "
                                 "TERMA voxel, 576 directions, every in-grid walk voxel), mean of "
                                 f"{min(args.update_beams, B)} beams of the workload, times beams/s"}

    # ---- extras: single-beam latency, plain scatter path, CPU baseline (rank 0)
    extras = {}
    if rank == 0 and not args.no_extras:
        lat = []
        for i in range(args.latency_beams):
            job = eng.job(ph, rho, beams[i][0], dblocks[i], SETTINGS, dose=doses[0])
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            eng.run(job)
            eng.sync()
            lat.append(1000.0 * (time.perf_counter() - t0))
        extras["single_beam_latency_ms"] = {"p50": percentile(lat, 0.5), "p99": percentile(lat, 0.99),
                                            "n": len(lat)}
        extras["single_beam_beams_per_s"] = 1000.0 / statistics.mean(lat)
        pl = []
        for i in range(args.plain_beams):
            job = eng.job(ph, rho, beams[i][0], dblocks[i], SETTINGS, dose=doses[0])
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            eng.run(job, scatter=True)
            eng.sync()
            pl.append(time.perf_counter() - t0)
        extras["plain_gpu_beams_per_s"] = len(pl) / sum(pl)
        extras["plain_gpu_path"] = "prologue + per-voxel scatter with float32 atomics, one beam per launch"
        extras["batching_ratios"] = {
            "batched_over_single_beam": value / extras["single_beam_beams_per_s"],
            "batched_over_plain_scatter": value / extras["plain_gpu_beams_per_s"],
            "target_read_against": "plain_gpu_beams_per_s: the reference's own structure (one beam per "
                                   "launch, per-voxel float32-atomic scatter) on the GPU; "
                                   "single_beam_beams_per_s is this engine's spectral path one beam per call"}
        if args.serve_requests > 0:
            extras["serving"] = serving_extras(args, dev)
        if args.adjoint_iters > 0:
            extras["adjoint"] = adjoint_extras(args, dev)
        if args.batch_beams > 0:
            extras["batched_captured"] = batched_extras(args, dev)
        if not args.no_cpu:
            cv, cores, dt = cpu_oracle_beams(ph, beams[:args.cpu_beams])
            extras["cpu_baseline"] = {
                "value": cv, "unit": "beams/s", "cores": cores, "kind": "port", "cpu": host_cpu(),
                "sample": f"{args.cpu_beams} whole beam(s) of the workload, FP64 oracle "
                          f"(C++ restatement of conehead's GPU path), OpenMP, {dt:.1f} s"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "beams/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * job_s / args.steps,
            "step_ms_spread": {"min": min(step_ms), "median": statistics.median(step_ms), "max": max(step_ms)},
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded slab phantom and beams; no dataset)",
            "config": config(args),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": traffic,
                         "kernel": (("spectral cone stage, plane path (spec_z_forward_plane, spec_plane, "
                                     "spec_z_inverse_plane)" if plane_path(ph.size) else
                                     "spectral cone stage (spec_z_forward, spec_y, spec_x, spec_y, spec_z_inverse)")
                                    if method == "spectral" else "cone_gather_kernel"),
                         "algorithmic_bytes_per_step": alg_bytes,
                         "algorithmic_basis": "8 N bytes per beam (TERMA read, dose write), N = grid voxels",
                         "traffic_over_algorithmic": traffic / alg_bytes if traffic else None,
                         "pass_bytes_per_step": pass_bytes,
                         "pass_traffic_frac": pass_bytes / (cone_ms * 1e-3) / 1e9 / hbm_peak,
                         "pass_basis": ("bytes the FFT pass structure must move (TERMA pair in, the A "
                                        "intermediate (and B on the five-pass path) written and read twice, "
                                        "dose pair out, S^ once per launch) over the stage time: how well the "
                                        "passes stream, not how close the stage is to its bound")
                                       if method == "spectral" else
                                       "as achieved",
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback"},
            "onchip": onchip,
            "cone_ms_per_step": cone_ms,
            "prologue_ms_per_step": statistics.mean(x["ms_prologue"] for x in stats),
            "range_ms_per_step": statistics.mean(x["ms_range"] for x in stats),
            "updates_per_step": updates,
            "e2e": e2e,
            "clocks": clk,
            "cone_method": method,
            "stages": stage_rooflines(stats, B, N, alg_bytes, cone_ms, hbm_peak, method),
            "updates": updates_line,
            "gpu_launches": args.steps * launches_per_step,
            "schedule": schedule,
        }
        line.update(extras)
        print(json.dumps(line))
    barrier()
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--beams", type=int, default=32, help="beams per step")
    ap.add_argument("--grid", type=int, default=128)
    ap.add_argument("--spacing", type=float, default=0.25)
    ap.add_argument("--field", type=float, default=5.0)
    ap.add_argument("--latency-beams", type=int, default=20)
    ap.add_argument("--plain-beams", type=int, default=2)
    ap.add_argument("--cpu-beams", type=int, default=2)
    ap.add_argument("--serve-requests", type=int, default=100, help="requests per serving rate (0: skip)")
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[50.0, 200.0, 2000.0])
    ap.add_argument("--serve-batch", type=int, default=32, help="beams per serving batch at most")
    ap.add_argument("--serve-no-warm", action="store_true", help="skip the serving executor's warm-up")
    ap.add_argument("--adjoint-iters", type=int, default=5, help="timed gradient evaluations (0: skip)")
    ap.add_argument("--batch-beams", type=int, default=64, help="beams of the captured mixed batch (0: skip)")
    ap.add_argument("--batch-iters", type=int, default=5)
    ap.add_argument("--no-autotune", action="store_true", help="time the default schedule")
    ap.add_argument("--update-beams", type=int, default=4,
                    help="beams sampled for the reference-equivalent updates/s (0: skip)")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only", choices=["serving", "adjoint", "batched"], default=None,
                    help="run one extra measurement alone and print its JSON (for profiling)")
    args = ap.parse_args(argv)
    args.warmup = max(3, args.warmup)      # at least three untimed warm-up steps
    if args.impl == "reference":
        return run_reference(args)
    if args.only:
        import torch
        dev = torch.device("cuda", 0)
        fn = {"serving": serving_extras, "adjoint": adjoint_extras, "batched": batched_extras}[args.only]
        print(json.dumps({args.only: fn(args, dev)}))
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
