"""Autotuner for the cone and TERMA schedule (``ch_tuning``).

The schedule knobs do not change results (beyond the float order of the
dose sums), only speed, and the best setting depends on the workload:
grid sizes, field sizes and how many beams share one cone launch.
``autotune`` times every candidate on a representative batch (CUDA events
on the engine's stream, after a warm-up) and keeps the fastest; results are
cached in a JSON file keyed by the device and a workload signature, so a
later call with a similar batch is free.

Knobs (see include/conehead_gb300.h):
  cone_method        0 = spectral (FFT convolution with the tap stencil),
                     1 = stencil gather
  dir_group          unique directions per gather work unit (16, 32, 64)
  unit_order         0 = a tile's direction groups run back to back,
                     1 = a direction group's tiles do
  terma_ctas_per_sm  CTAs per SM of the TERMA pass (2, 3; the batched pass is
                     persistent and holds at most 3 per SM, its register
                     budget, so larger values run as 3)
"""
import json
import os
import statistics

import numpy as np

DEFAULT = {"dir_group": 16, "unit_order": 0, "terma_ctas_per_sm": 8, "cone_method": 0}
# Units of more than 64 directions also run, but every thread then sums more
# taps in one float32 register before its add to the dose: measured against
# the float32-mirrored oracle at 64^3 the error grows from 5e-7 of Dmax (16
# or 32 directions) and 9e-7 (64) to 1.6e-6 (128) and 9e-6 (1024).  The tuner
# stays at 64 or below, where the precision is unchanged.
CANDIDATES = ([{"dir_group": 16, "unit_order": 0, "terma_ctas_per_sm": t, "cone_method": 0} for t in (2, 3)] +
              [{"dir_group": g, "unit_order": o, "terma_ctas_per_sm": t, "cone_method": 1}
               for g in (16, 32, 64) for o in (0, 1) for t in (2, 3)])


def cache_path():
    return os.environ.get("CONEHEAD_GB300_TUNING",
                          os.path.join(os.path.expanduser("~"), ".cache", "conehead_gb300", "tuning.json"))


def signature(device_name, jobs):
    """Device + spacing + grid-size histogram + beam count (bucketed) + mean open area (bucketed)."""
    sizes = {}
    area = []
    spacing = None
    for j in jobs:
        n = tuple(int(j.grid.n[k]) for k in range(3))
        sizes[n] = sizes.get(n, 0) + 1
        spacing = tuple(round(float(j.grid.spacing[k]), 4) for k in range(3))
        area.append(j.beam.block_rows * j.beam.block_cols)
    n_beams = len(jobs)
    beams_bucket = 1 << max(0, int(np.ceil(np.log2(max(n_beams, 1)))))
    area_bucket = int(np.round(np.log2(max(np.mean(area), 1.0)))) if area else 0
    hist = ",".join(f"{n[0]}x{n[1]}x{n[2]}:{round(c / n_beams, 2)}" for n, c in sorted(sizes.items()))
    return f"{device_name}|{spacing}|{hist}|beams~{beams_bucket}|area~2^{area_bucket}"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(path, table):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def time_batch(engine, jobs, iters=2, warmup=1):
    """Median ms of run_batch(jobs) (CUDA events on the engine's stream)."""
    import torch
    st = torch.cuda.current_stream(engine.device)
    for _ in range(warmup):
        engine.run_batch(jobs)
    ms = []
    for _ in range(iters):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        engine.run_batch(jobs)
        e1.record(st)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    engine.sync()
    return statistics.median(ms)


def autotune(engine, jobs, candidates=None, iters=2, force=False, path=None, timer=None, device_name=None):
    """Pick and set the fastest schedule for this batch; returns
    {"tuning": best, "ms": its time, "table": [(candidate, ms)...], "cached": bool}.
    ``timer(engine, jobs)`` -> ms replaces the CUDA-event timing (tests)."""
    path = path or cache_path()
    if device_name is None:
        import torch
        device_name = torch.cuda.get_device_name(engine.device)
    timer = timer or (lambda e, j: time_batch(e, j, iters=iters))
    key = signature(device_name, jobs)
    table = _load(path)
    if not force and key in table:
        best = {**DEFAULT, **table[key]["tuning"]}
        engine.set_tuning(**best)
        return {"tuning": best, "ms": table[key]["ms"], "table": table[key].get("table", []), "cached": True}
    results = []
    for cand in candidates or CANDIDATES:
        cand = {**DEFAULT, **cand}          # every knob named, unnamed ones at their defaults
        engine.set_tuning(**cand)
        results.append((cand, timer(engine, jobs)))
    best, ms = min(results, key=lambda r: r[1])
    engine.set_tuning(**best)
    table[key] = {"tuning": best, "ms": ms, "table": [[c, m] for c, m in results]}
    _save(path, table)
    return {"tuning": best, "ms": ms, "table": results, "cached": False}
