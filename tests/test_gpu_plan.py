"""GPU: the MLC block map rasterised on the device, and plan dose.

* ``ch_block_from_mlc`` writes exactly the host map's cells (bit for bit)
  for the reference's plan fixture and the seeded synthetic plans, for the
  jaw opening and for windows that run off the map.
* A dose from ``Block(plan=...)`` through the device rasteriser has the
  same blocked fraction and TERMA, bit for bit, as the same map uploaded
  from the host, the same dose up to float atomic order, and stays within
  the dose bars of the fp32-mirrored and FP64 oracles.
* A multi-beam plan in one batched call equals the beams one at a time.
"""
import ctypes
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
from make_golden import _plan_ns, synthetic_plans  # noqa: E402

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(GOLDEN, "RP.3DCRT.dcm")
DOSE_BAR = 5e-3
DOSE_F32 = 2e-4


@pytest.fixture(scope="module")
def eng():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conehead_gb300.build import build
    build()
    from conehead_gb300.conehead import engine
    return engine(0)


def _plans():
    from conehead_gb300 import dicom
    out = {"fixture": dicom.read(FIXTURE, force=True)}
    for name, d in synthetic_plans().items():
        out[name] = _plan_ns(d)
    return out


def _raster(eng, mlc, r0, r1, c0, c1):
    import torch
    from conehead_gb300 import _native as N
    out = torch.full((r1 - r0, c1 - c0), -7.0, dtype=torch.float32, device=eng.device)
    m = mlc.struct()
    N.check(eng.L.ch_block_from_mlc(ctypes.byref(m), out.data_ptr(), r1 - r0, c1 - c0, r0, c0, eng.stream()),
            "ch_block_from_mlc")
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_device_raster_equals_host_map(eng):
    from conehead_gb300.block import MLCField
    for name, plan in _plans().items():
        mlc = MLCField.from_plan(plan)
        full = mlc.values()
        r0, r1, c0, c1 = mlc.window
        if r1 > r0 and c1 > c0:
            got = _raster(eng, mlc, r0, r1, c0, c1)
            assert np.array_equal(got, full[r0:r1, c0:c1]), name
        # a window hanging over every edge of the map reads 0 outside it
        lo_r, lo_c = -5, -9
        got = _raster(eng, mlc, lo_r, mlc.rows + 6, lo_c, 4000 + 3)
        expect = np.zeros_like(got)
        expect[-lo_r:-lo_r + mlc.rows, -lo_c:-lo_c + 4000] = full
        assert np.array_equal(got, expect), name


def test_engine_upload_mlc_matches_crop_path(eng):
    from conehead_gb300.block import Block
    blk = Block(plan=_plans()["fixture"])
    db = eng.upload_mlc(blk.mlc)
    full = blk.mlc.values()
    crop = db.crop.cpu().numpy()
    assert (db.r0, db.c0, db.full_shape) == (1590, 1660, (4000, 4000))
    assert np.array_equal(crop, full[db.r0:db.r0 + crop.shape[0], db.c0:db.c0 + crop.shape[1]])
    # outside the crop the host map is zero, as the crop convention needs
    outside = full.copy()
    outside[db.r0:db.r0 + crop.shape[0], db.c0:db.c0 + crop.shape[1]] = 0
    assert not outside.any()


def _dose_error(d, ref):
    dmax = ref.max()
    mask = ref > 0.01 * dmax
    return np.abs(d.astype(np.float64) - ref)[mask].max() / dmax


def test_plan_dose_device_map_equals_host_map_and_oracle(eng, settings, oracle_lib):
    from conehead_gb300 import Block, Conehead, Source
    from conehead_gb300.phantoms import slab_phantom
    ph = slab_phantom(48, 0.4, seed=9, n_inserts=6)
    plan = _plans()["fixture"]
    src = Source()
    src.gantry = 30
    src.collimator = 15
    blk = Block(plan=plan)
    assert blk.device_mlc() is not None
    out = Conehead().calculate(src, blk, ph, settings, return_intermediates=True)
    assert blk.device_mlc() is not None            # the dose path never built the host map
    host = Block(plan=plan)
    _ = host.block_values                           # materialised: the engine uploads the map
    out_host = Conehead().calculate(src, host, ph, settings, return_intermediates=True)
    for k in ("blocked", "terma"):
        assert np.array_equal(out[k], out_host[k]), k
    # dose sums each voxel's work units with float atomics in arrival order
    assert np.abs(out["dose"] - out_host["dose"]).max() <= 1e-5 * out_host["dose"].max()
    assert out["dose"].max() > 0
    ref = oracle_lib.calculate(src, host, ph, settings, oracle_lib.MODE_F32)
    assert np.array_equal(out["blocked"], ref["blocked"])
    e32 = _dose_error(out["dose"], ref["dose"])
    ref64 = oracle_lib.calculate(src, host, ph, settings, oracle_lib.MODE_F64)
    e64 = _dose_error(out["dose"], ref64["dose"])
    print(f"plan fixture 48^3: vs fp32 oracle {e32:.2e}, vs FP64 oracle {e64:.2e} of Dmax")
    assert e32 <= DOSE_F32 and e64 <= DOSE_BAR


def test_multi_beam_plan_batch_equals_single(eng, settings):
    import types
    from conehead_gb300 import Conehead
    from conehead_gb300.phantoms import slab_phantom
    from conehead_gb300.plan import plan_beams
    ph = slab_phantom(64, 0.3, seed=4, n_inserts=5)
    ns = types.SimpleNamespace
    d = synthetic_plans()
    beams_ns = []
    rng = np.random.default_rng(8)
    for name in ("millennium_random", "agility_collide", "fixture_like"):
        if name == "fixture_like":
            beams_ns.append(_plans()["fixture"].BeamSequence[0])
            continue
        b = _plan_ns(d[name]).BeamSequence[0]
        b.ControlPointSequence[0].GantryAngle = float(rng.uniform(0, 360))
        b.ControlPointSequence[0].BeamLimitingDeviceAngle = float(rng.uniform(0, 90))
        b.SourceAxisDistance = 1000.0
        beams_ns.append(b)
    plan = ns(BeamSequence=beams_ns)
    pairs = plan_beams(plan)
    assert all(blk.device_mlc() is not None for _, blk in pairs)
    ch = Conehead()
    batch = ch.calculate_batch(pairs, ph, settings)
    for (src, blk), db in zip(pairs, batch):
        single = ch.calculate(src, blk, ph, settings)
        assert db.max() > 0
        assert np.abs(db - single).max() <= 1e-5 * single.max()
