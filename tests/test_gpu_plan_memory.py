"""GPU: the plan's memory queries used for admission control.

* ``ch_plan_memory`` splits tables (kernel, stencils) from the scratch arena;
* ``ch_batch_scratch_bytes`` says how much a batch needs and how much the
  arena would grow: nothing for a batch it has already run, all of it after a
  trim;
* ``ch_plan_trim`` gives the arena back and the next dose still works.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conehead_gb300.build import build
    build()


def _mem(eng):
    from conehead_gb300 import _native as N
    t, s = ctypes.c_size_t(), ctypes.c_size_t()
    N.check(eng.L.ch_plan_memory(eng.plan, ctypes.byref(t), ctypes.byref(s)), "ch_plan_memory")
    return t.value, s.value


def _need(eng, jobs):
    from conehead_gb300 import _native as N
    grids = (N.Grid * len(jobs))(*[j.grid for j in jobs])
    g, t = ctypes.c_size_t(), ctypes.c_size_t()
    N.check(eng.L.ch_batch_scratch_bytes(eng.plan, len(jobs), grids, ctypes.byref(g), ctypes.byref(t)),
            "ch_batch_scratch_bytes")
    return g.value, t.value


def test_memory_queries_and_trim(gpu, settings):
    from conehead_gb300 import _native as N
    from conehead_gb300.engine import DoseEngine
    from conehead_gb300.phantoms import random_beam, slab_phantom
    eng = DoseEngine(0)
    eng.set_kernel(settings["energy_weights"])
    eng.prepare((48, 48, 48), (0.25, 0.25, 0.25))
    tables, scratch = _mem(eng)
    assert tables > 1 << 20 and scratch == 0            # K (2.3 MB) + stencils, no arena yet
    ph = slab_phantom(48, 0.25, seed=2, n_inserts=3)
    rho = eng.upload_densities(ph.densities)
    rng = np.random.default_rng(2)
    jobs = [eng.job(ph, rho, s, eng.block_for(b), settings) for s, b in (random_beam(rng) for _ in range(3))]
    growth, total = _need(eng, jobs)
    assert growth == total > 48 ** 3 * 4 * 3            # at least the three TERMA volumes
    eng.run_batch(jobs)
    eng.sync()
    ref = [j.dose.cpu().numpy().copy() for j in jobs]
    assert _mem(eng) == (tables, total)
    assert _need(eng, jobs) == (0, total)               # a batch it has run needs no growth
    assert _need(eng, jobs[:1])[0] == 0                 # nor does a smaller one
    N.check(eng.L.ch_plan_trim(eng.plan), "ch_plan_trim")
    assert _mem(eng) == (tables, 0)
    assert _need(eng, jobs) == (total, total)
    eng.run_batch(jobs)
    eng.sync()
    for j, r in zip(jobs, ref):
        assert np.abs(j.dose.cpu().numpy() - r).max() <= 1e-5 * r.max()
    eng.close()
