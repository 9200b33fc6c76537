"""GPU: the physics extensions, flagged in the settings dict.

* coneDistance = "radiological": equal to the reference in water; in a
  heterogeneous phantom equal to the oracle's radiological cone applied to
  the GPU's own TERMA, and different from the reference.
* coneFrame = "beam": equal to the reference at gantry = collimator = 0;
  for a turned beam equal to the oracle's cones rotated by the beam's
  orientation, and different from the reference.
* Beams with and without options mix in one batch; captured batches, the
  static entry point and the adjoint refuse options.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 2e-4      # of Dmax, as the float32-mirrored oracle comparisons


@pytest.fixture(scope="module")
def eng():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conehead_gb300.build import build
    build()
    from conehead_gb300.conehead import engine
    return engine(0)


def _beam(g, c, field=(-2.5, 3.0, -2.0, 2.5)):
    from conehead_gb300 import Block, Source
    src = Source()
    src.gantry = g
    src.collimator = c
    blk = Block()
    blk.set_rect(*field)
    return src, blk


def _calc(src, blk, ph, settings, **opts):
    from conehead_gb300 import Conehead
    return Conehead().calculate(src, blk, ph, dict(settings, **opts), return_intermediates=True)


def _err(d, ref):
    return np.abs(d.astype(np.float64) - ref).max() / ref.max()


def test_radiological_distance(eng, settings, oracle_lib):
    from conehead_gb300.kernel import poly_kernel_tables
    from conehead_gb300.phantoms import slab_phantom, water_phantom
    src, blk = _beam(30.0, 0.0)
    w = water_phantom(24, 0.5)
    a = _calc(src, blk, w, settings)["dose"]
    b = _calc(src, blk, w, settings, coneDistance="radiological")["dose"]
    # the same taps and weights; only the summation differs (per-source float
    # atomics against the stencil gather's per-output sums)
    assert _err(b, a) <= 2e-5
    ph = slab_phantom(32, 0.5, seed=4, n_inserts=4)
    out = _calc(src, blk, ph, settings, coneDistance="radiological")
    ref_geo = _calc(src, blk, ph, settings)["dose"]
    K, th, phs = poly_kernel_tables(settings["energy_weights"])
    swap = ph.size[0] == ph.size[1]
    ref = oracle_lib.cone_ext(out["terma"], ph.size, ph.spacing, K, th, phs, oracle_lib.MODE_F32,
                              rho=ph.densities, swap_xy=swap)
    e = _err(out["dose"], ref)
    print(f"radiological distance 32^3: vs oracle {e:.2e} of Dmax; vs geometric {_err(out['dose'], ref_geo):.2e}")
    assert e <= TOL
    assert _err(out["dose"], ref_geo) > 1e-2


def test_cones_in_beam_frame(eng, settings, oracle_lib):
    from conehead_gb300.kernel import poly_kernel_tables
    from conehead_gb300.phantoms import slab_phantom
    ph = slab_phantom(32, 0.5, seed=5, n_inserts=4)
    src0, blk0 = _beam(0.0, 0.0)
    a = _calc(src0, blk0, ph, settings)["dose"]
    b = _calc(src0, blk0, ph, settings, coneFrame="beam")["dose"]
    assert _err(b, a) <= 1e-6
    src, blk = _beam(60.0, 30.0)
    out = _calc(src, blk, ph, settings, coneFrame="beam")
    room = _calc(src, blk, ph, settings)["dose"]
    K, th, phs = poly_kernel_tables(settings["energy_weights"])
    ref = oracle_lib.cone_ext(out["terma"], ph.size, ph.spacing, K, th, phs, oracle_lib.MODE_F32,
                              frame=np.asarray(src.transform, dtype=np.float64))
    e = _err(out["dose"], ref)
    print(f"beam-frame cones G60 C30: vs oracle {e:.2e} of Dmax; vs room frame {_err(out['dose'], room):.2e}")
    assert e <= TOL
    assert _err(out["dose"], room) > 1e-3


def test_mixed_batch_and_refusals(eng, settings):
    import ctypes
    import torch
    from conehead_gb300 import _native as N
    from conehead_gb300.phantoms import slab_phantom
    ph = slab_phantom(32, 0.5, seed=6, n_inserts=3)
    rho = eng.upload_densities(ph.densities)
    beams = [_beam(10.0, 0.0), _beam(70.0, 20.0), _beam(200.0, 45.0)]
    opts = [{}, {"coneFrame": "beam"}, {"coneDistance": "radiological", "coneFrame": "beam"}]
    jobs = [eng.job(ph, rho, s, eng.block_for(b), dict(settings, **o)) for (s, b), o in zip(beams, opts)]
    eng.run_batch(jobs)
    eng.sync()
    batch = [j.dose.cpu().numpy().copy() for j in jobs]
    for (s, b), o, d in zip(beams, opts, batch):
        single = _calc(s, b, ph, settings, **o)["dose"]
        assert _err(d, single) <= 1e-5
    with pytest.raises(N.CHError, match="reference physics"):
        eng.capture(jobs)
    job = jobs[1]
    st = eng.L.ch_dose_static(eng.plan, ctypes.byref(job.grid), job.rho.data_ptr(), job.swap_xy,
                              ctypes.byref(job.beam), ctypes.byref(job.settings), job.dose.data_ptr(), eng.stream())
    assert st == 1 and "reference physics" in eng.L.ch_last_error().decode()
