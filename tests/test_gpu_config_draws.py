"""GPU parity on draws of the batched, served and spectrum-switch layers,
against the CPU oracle (float32-mirrored and FP64).

* Batched: beams drawn as the batched workload draws them -- slab phantoms
  of 64^3, 96^3, 128^3 and 160^3 at 0.25 cm, jaws X and Y each uniform in
  [2, 20] cm, gantry U[0, 360), collimator U[0, 90) -- with the 160^3 grid
  (FFT period 384) and the 96^3 grid (period 192) both present; the 128^3
  and 160^3 draws cap the jaws at 12 cm to keep the FP64 oracle affordable.
  The same beams run as one ch_dose_batch call and as one captured CUDA
  graph (ch_batch_create / ch_batch_launch), and every dose of both is
  compared with the oracle: the cone stage is
  conehead/conehead.py:385-488, blocking of large rotated fields :71-120.
* Served: a request on a 192^3 phantom (period 384, the largest grid of the
  serving workload) through DoseServer, compared with the oracle.
* Spectrum switch: after ch_plan_set_kernel reweights the resident tap
  stencils in place to a harder spectrum (no stencil rebuild), the dose
  equals the oracle run with that spectrum (conehead/kernel.py:27-72).
"""
import numpy as np
import pytest

from oracle_checks import check_dose

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
    return torch


def _draws():
    """Four beams drawn like the batched workload: (grid n, source, block,
    jaw sizes in cm)."""
    from conehead_gb300 import Block, Source
    rng = np.random.default_rng(2047)      # draws a 96^3 field of 18.8 x 12.3 cm
    out = []
    for n, hi in ((160, 12.0), (96, 20.0), (128, 12.0), (64, 20.0)):
        src = Source()
        src.gantry = float(rng.uniform(0.0, 360.0))
        src.collimator = float(rng.uniform(0.0, 90.0))
        fx, fz = rng.uniform(2.0, hi, size=2)
        blk = Block()
        blk.set_rect(-fx / 2, fx / 2, -fz / 2, fz / 2)
        out.append((n, src, blk, (fx, fz)))
    return out


def test_batched_draws_match_the_oracle(gpu, settings, oracle_lib):
    from conehead_gb300.engine import DoseEngine
    from conehead_gb300.phantoms import slab_phantom
    torch = gpu
    draws = _draws()
    phantoms = {n: slab_phantom(n, 0.25, seed=n) for n, _, _, _ in draws}
    eng = DoseEngine(0)
    try:
        eng.set_kernel(settings["energy_weights"])
        rhos = {n: eng.upload_densities(ph.densities) for n, ph in phantoms.items()}
        blocks = [eng.block_for(blk) for _, _, blk, _ in draws]
        eng.prepare((160, 160, 160), (0.25, 0.25, 0.25))
        jobs = [eng.job(phantoms[n], rhos[n], src, db, settings) for (n, src, _, _), db in zip(draws, blocks)]
        eng.run_batch(jobs)
        eng.sync()
        batched = [j.dose.cpu().numpy().copy() for j in jobs]
        # the same beams captured into one graph, into fresh outputs
        cap_jobs = [eng.job(phantoms[n], rhos[n], src, db, settings,
                            dose=torch.full(tuple(phantoms[n].size), -1.0, device=eng.device))
                    for (n, src, _, _), db in zip(draws, blocks)]
        batch = eng.capture(cap_jobs)
        batch.launch()
        batch.sync()
        captured = [j.dose.cpu().numpy().copy() for j in cap_jobs]
        batch.close()
    finally:
        eng.close()
    for (n, src, blk, (fx, fz)), d_b, d_c in zip(draws, batched, captured):
        label = f"{n}^3 gantry {src.gantry:.1f} collimator {src.collimator:.1f} jaws {fx:.1f} x {fz:.1f} cm"
        # captured replay: the same kernels in the same order
        assert np.abs(d_c - d_b).max() <= 1e-5 * d_b.max()
        check_dose(oracle_lib, {"batched " + label: d_b, "captured " + label: d_c}, src, blk, phantoms[n],
                   settings, label, f64=True)


def test_served_192_beam_matches_the_oracle(gpu, settings, oracle_lib):
    from conehead_gb300.phantoms import random_beam, slab_phantom
    from conehead_gb300.serving import DoseServer, GpuExecutor, Request
    ph = slab_phantom(192, 0.25, seed=192, n_inserts=12)
    ex = GpuExecutor(0, n_slots=2)
    try:
        ex.add_phantom("p192", ph)
        ex.prepare(settings, (0.25, 0.25, 0.25), (192, 192, 192))
        rng = np.random.default_rng(192)
        beams = [random_beam(rng, field=5.0), random_beam(rng, rect=(2.0, 8.0), collimator=True)]
        server = DoseServer(ex, budget_bytes=16 << 30, max_wave_beams=8)
        req = server.submit(Request("p192", beams, settings))
        server.run()
        assert req.error is None, req.error
        doses = [d.numpy().copy() for d in req.doses]
    finally:
        ex.close()
    for (src, blk), d in zip(beams, doses):
        check_dose(oracle_lib, d, src, blk, ph, settings, f"served 192^3 gantry {src.gantry:.1f}", f64=True)


def test_reweighted_spectrum_matches_the_oracle(gpu, settings, oracle_lib):
    from conehead_gb300.engine import DoseEngine
    from conehead_gb300.phantoms import random_beam, slab_phantom
    ph = slab_phantom(64, 0.25, seed=61, n_inserts=6)
    rng = np.random.default_rng(61)
    src, blk = random_beam(rng, rect=(3.0, 10.0), collimator=True)
    hard = dict(settings, energy_weights=HARD)
    eng = DoseEngine(0)
    try:
        rho = eng.upload_densities(ph.densities)
        eng.set_kernel(settings["energy_weights"])
        eng.run(eng.job(ph, rho, src, eng.block_for(blk), settings))      # builds the stencils
        eng.sync()
        eng.set_kernel(HARD)                                               # reweights them in place
        d = eng.run(eng.job(ph, rho, src, eng.block_for(blk), hard))
        eng.sync()
        d = d.cpu().numpy()
    finally:
        eng.close()
    check_dose(oracle_lib, d, src, blk, ph, hard, "reweighted spectrum 64^3", f64=True)
