"""GPU: captured batches (one CUDA graph per batch) and the schedule knobs.

* A captured batch of beams on mixed grids, jaw rectangles, gantry and
  collimator angles gives the doses of ch_dose_batch; replays recompute from
  the current densities (changed in place between launches).
* Every schedule the autotuner can pick gives the same dose.
* While a captured batch exists the plan refuses new kernel tables, and the
  autotuner runs end to end on the device.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def setup(settings):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conehead_gb300.build import build
    build()
    from conehead_gb300.engine import DoseEngine
    from conehead_gb300.phantoms import random_beam, slab_phantom
    eng = DoseEngine(0)
    eng.set_kernel(settings["energy_weights"])
    rng = np.random.default_rng(41)
    phantoms = {n: slab_phantom(n, 0.25, seed=n, n_inserts=4) for n in (32, 48, 64)}
    rhos = {n: eng.upload_densities(ph.densities) for n, ph in phantoms.items()}
    jobs = []
    for i in range(9):
        n = (32, 48, 64)[i % 3]
        src, blk = random_beam(rng, rect=(2.0, 12.0), collimator=True)
        jobs.append(eng.job(phantoms[n], rhos[n], src, eng.block_for(blk), settings))
    eng.prepare((64, 64, 64), (0.25, 0.25, 0.25))
    yield eng, jobs, phantoms, rhos
    eng.close()


def _doses(eng, jobs):
    eng.run_batch(jobs)
    eng.sync()
    return [j.dose.cpu().numpy().copy() for j in jobs]


def _close(a, b):
    return all(np.abs(x - y).max() <= TOL * max(y.max(), 1e-30) for x, y in zip(a, b))


def test_captured_batch_matches_and_replays(setup):
    import torch
    eng, jobs, phantoms, rhos = setup
    eng.set_tuning()
    ref = _doses(eng, jobs)
    assert all(r.max() > 0 for r in ref)
    batch = eng.capture(jobs)
    try:
        for j in jobs:
            j.dose.fill_(-1.0)
        batch.launch()
        batch.sync()
        got = [j.dose.cpu().numpy().copy() for j in jobs]
        assert _close(got, ref)
        batch.launch()
        batch.sync()
        assert _close([j.dose.cpu().numpy() for j in jobs], ref)
        # densities change in place: the replay follows them
        rhos[48].mul_(1.3)
        batch.launch()
        batch.sync()
        got2 = [j.dose.cpu().numpy().copy() for j in jobs]
    finally:
        batch.close()
    ref2 = _doses(eng, jobs)
    rhos[48].div_(1.3)
    assert _close(got2, ref2)
    changed = [i for i in range(len(jobs)) if int(jobs[i].grid.n[0]) == 48]
    assert all(np.abs(got2[i] - ref[i]).max() > 1e-3 * ref[i].max() for i in changed)


def test_every_schedule_gives_the_same_dose(setup):
    from conehead_gb300.autotune import CANDIDATES
    eng, jobs, _, _ = setup
    eng.set_tuning()
    ref = _doses(eng, jobs)
    for cand in CANDIDATES:
        eng.set_tuning(**cand)
        assert _close(_doses(eng, jobs), ref), cand
    eng.set_tuning()


def test_plan_is_frozen_while_a_batch_lives_and_autotune_runs(setup, settings, tmp_path):
    from conehead_gb300 import _native as N
    from conehead_gb300.autotune import autotune
    eng, jobs, _, _ = setup
    batch = eng.capture(jobs[:3])
    try:
        eng._kernel_key = None                      # force a real ch_plan_set_kernel
        with pytest.raises(N.CHError, match="captured"):
            eng.set_kernel(settings["energy_weights"])
    finally:
        batch.close()
    eng.set_kernel(settings["energy_weights"])
    r = autotune(eng, jobs, candidates=[{"dir_group": 16, "unit_order": 0, "terma_ctas_per_sm": 8},
                                        {"dir_group": 32, "unit_order": 1, "terma_ctas_per_sm": 4}],
                 path=str(tmp_path / "t.json"))
    assert not r["cached"] and r["ms"] > 0 and eng.get_tuning() == r["tuning"]
    assert autotune(eng, jobs, path=str(tmp_path / "t.json"))["cached"]
    eng.set_tuning()
