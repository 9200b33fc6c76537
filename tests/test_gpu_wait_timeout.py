"""GPU: a bounded device-side wait that expires is reported, and the plan
stays usable.

The gather cone stage runs a producer warp (TMA window copies into two
shared-memory slots) and consumer warps, synchronised by mbarriers.  Every
wait of that pipeline is bounded.  When one gives up, the kernel records
the failure, lets its own copies in flight land (a wait with the full
default bound) and returns, so no trap, fault or hang is involved.  The test
hook ``ch_plan_set_wait_limit(plan, iterations, withhold)`` makes a wait
run out with nothing broken: with ``withhold`` = 1 the producer issues no
window (every consumer's wait expires), with 2 the consumers never free a
slot (the producer's wait expires while two window copies are in flight).
``ch_plan_sync`` must report CH_ERR_TIMEOUT, and the next call with the hook
off must give the normal dose.

The reference has no device-side waits; its only device-side failure, a
ray parallel to the blocking plane (conehead/conehead.py:34-35), is tested
in test_gpu_parity.py.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CH_ERR_TIMEOUT = 4


@pytest.fixture(scope="module")
def eng(settings):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conehead_gb300.build import build
    build()
    from conehead_gb300.engine import DoseEngine
    e = DoseEngine(0)
    e.set_kernel(settings["energy_weights"])
    e.set_tuning(cone_method=1)           # the gather: the stage with the pipeline waits
    yield e
    e.close()


@pytest.mark.parametrize("withhold", [1, 2], ids=["no-window", "no-free-slot"])
def test_expired_wait_reports_timeout_and_the_plan_recovers(eng, settings, withhold):
    from conehead_gb300 import _native as N
    from conehead_gb300.phantoms import random_beam, slab_phantom
    ph = slab_phantom(48, 0.25, seed=48, n_inserts=4)
    rng = np.random.default_rng(48)
    src, blk = random_beam(rng, field=6.0)
    rho = eng.upload_densities(ph.densities)
    db = eng.block_for(blk)
    ref = eng.run(eng.job(ph, rho, src, db, settings)).clone()
    eng.sync()
    ref = ref.cpu().numpy()
    assert ref.max() > 0
    # a short bound (the waits that cannot complete end in about a
    # millisecond) and the withheld arrivals
    eng.set_wait_limit(1 << 12, withhold)
    try:
        eng.run(eng.job(ph, rho, src, db, settings))
        with pytest.raises(N.CHError) as err:
            eng.sync()
        assert err.value.status == CH_ERR_TIMEOUT
        assert "bounded device wait" in str(err.value)
    finally:
        eng.set_wait_limit(0, 0)
    # the plan and the context are fine: the next call gives the normal dose
    d = eng.run(eng.job(ph, rho, src, db, settings))
    eng.sync()
    d = d.cpu().numpy()
    assert np.abs(d - ref).max() <= 1e-5 * ref.max()


def test_wait_limit_hook_rejects_unknown_modes(eng):
    from conehead_gb300 import _native as N
    with pytest.raises(N.CHError):
        eng.set_wait_limit(0, 3)
