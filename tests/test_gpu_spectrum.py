"""GPU: switching the spectrum reweights the resident stencils.

A plan keeps its direction stencils across ``ch_plan_set_kernel`` calls that
keep the cone directions: only the tap weights (the per-direction kernel
increments) are recomputed on the device.  The dose after a switch must
equal the dose of a plan built from scratch for that spectrum, and
switching back must give the first dose again.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HARD = {"0.5": 0.03, "1.0": 0.06, "1.5": 0.08, "2.0": 0.09, "2.5": 0.09, "3.0": 0.09,
        "3.5": 0.08, "4.0": 0.08, "4.5": 0.07, "5.0": 0.06, "5.5": 0.05, "6.0": 0.04}


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conehead_gb300.build import build
    build()


def _dose(eng, ph, rho, beams, settings):
    jobs = [eng.job(ph, rho, s, eng.block_for(b), settings) for s, b in beams]
    eng.run_batch(jobs)
    eng.sync()
    return [j.dose.cpu().numpy().copy() for j in jobs]


def test_spectrum_switch_equals_fresh_build(gpu, settings):
    import torch
    from conehead_gb300.engine import DoseEngine
    from conehead_gb300.phantoms import random_beam, slab_phantom
    soft = dict(settings)
    hard = dict(settings, energy_weights=HARD)
    ph = slab_phantom(64, 0.25, seed=6, n_inserts=5)
    rng = np.random.default_rng(6)
    beams = [random_beam(rng, rect=(3.0, 9.0), collimator=True) for _ in range(3)]
    a = DoseEngine(0)
    rho = a.upload_densities(ph.densities)
    a.set_kernel(soft["energy_weights"])
    d_soft = _dose(a, ph, rho, beams, soft)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    a.set_kernel(hard["energy_weights"])          # stencils exist: reweight in place
    t_switch = time.perf_counter() - t0
    d_hard = _dose(a, ph, rho, beams, hard)
    b = DoseEngine(0)
    b.set_kernel(hard["energy_weights"])
    t0 = time.perf_counter()
    b.prepare((64, 64, 64), (0.25, 0.25, 0.25))   # full stencil build
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    d_fresh = _dose(b, ph, rho, beams, hard)
    print(f"spectrum switch {1e3 * t_switch:.1f} ms (host kernel tables included) vs stencil build "
          f"{1e3 * t_build:.1f} ms")
    for x, y in zip(d_hard, d_fresh):
        assert np.abs(x - y).max() <= 1e-6 * y.max()
    for x, y in zip(d_hard, d_soft):
        assert np.abs(x - y).max() > 1e-3 * y.max()   # the spectrum does matter
    a.set_kernel(soft["energy_weights"])
    for x, y in zip(_dose(a, ph, rho, beams, soft), d_soft):
        assert np.abs(x - y).max() <= 1e-6 * y.max()
    a.close()
    b.close()
