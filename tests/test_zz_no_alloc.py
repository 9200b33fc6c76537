"""ch_dose_static: the dose entry point that allocates nothing.

It serves callers that cannot call cudaMalloc. Examples are a host framework
that owns the device allocator, or code that must not allocate once it is set
up. Its scratch lives in a fixed device array inside the library. These tests
call it through the C ABI and check its dose against ordinary ch_dose on the
same inputs, on consecutive calls. They also check that device memory stays
put across calls, and that a grid too big for the array is refused with a
clear error.

This file is named so pytest collects it last. It builds its own plan, so it
passes alone in a fresh process and after every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5        # fraction of Dmax, the same bound as batch-vs-single


@pytest.fixture(scope="module")
def setup():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conehead_gb300.build import build
    build()
    from conehead_gb300.engine import DoseEngine
    eng = DoseEngine(0)
    from conftest import EXAMPLE_SETTINGS
    eng.set_kernel(EXAMPLE_SETTINGS["energy_weights"])
    yield eng, EXAMPLE_SETTINGS
    eng.close()


def call_static(eng, job):
    from conehead_gb300 import _native as N
    st = eng.L.ch_dose_static(eng.plan, ctypes.byref(job.grid), job.rho.data_ptr(), job.swap_xy,
                              ctypes.byref(job.beam), ctypes.byref(job.settings), job.dose.data_ptr(),
                              eng.stream())
    N.check(st, "ch_dose_static")


def test_static_matches_ch_dose_on_consecutive_calls(setup):
    import torch
    from conehead_gb300.phantoms import random_beam, slab_phantom
    eng, settings = setup
    rng = np.random.default_rng(21)
    ph = slab_phantom(64, 0.25, seed=21)
    rho = eng.upload_densities(ph.densities)
    beams = [random_beam(rng, rect=(3.0, 9.0), collimator=True) for _ in range(2)]
    blocks = [eng.upload_block(b.block_values) for _, b in beams]
    # ordinary path first: it also prepares the plan (stencils for 0.25 cm)
    refs = []
    for (src, _), db in zip(beams, blocks):
        refs.append(eng.run(eng.job(ph, rho, src, db, settings)).clone())
        eng.sync()
    refs = [r.cpu().numpy() for r in refs]
    assert all(r.max() > 0 for r in refs)
    outs = [torch.empty(ph.size, dtype=torch.float32, device=eng.device) for _ in range(3)]
    jobs = [eng.job(ph, rho, beams[0][0], blocks[0], settings, dose=outs[0]),
            eng.job(ph, rho, beams[1][0], blocks[1], settings, dose=outs[1]),
            eng.job(ph, rho, beams[0][0], blocks[0], settings, dose=outs[2])]
    call_static(eng, jobs[0])            # first call on this device: looks up the array
    eng.sync()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(eng.index)[0]
    call_static(eng, jobs[1])            # two more calls in a row, different beams
    call_static(eng, jobs[2])
    eng.sync()
    free_after = torch.cuda.mem_get_info(eng.index)[0]
    assert free_after == free_before
    for out, ref in zip([outs[0], outs[1], outs[2]], [refs[0], refs[1], refs[0]]):
        d = out.cpu().numpy()
        assert np.abs(d - ref).max() <= TOL * ref.max()


@pytest.mark.parametrize("size", [(48, 40, 37), (44, 44, 30)], ids=["ragged-swap0", "square-xy-swap1"])
def test_static_matches_ch_dose_on_smaller_grids(setup, size):
    """A plan prepared for 64^3 serves smaller, non-cubic grids: its tile
    count, z padding and scratch layout follow the grid of each call.  A grid
    with unequal x and y reads the densities as they are (swap_xy = 0); a
    square x/y grid reads them transposed, as the reference's resampling
    does (swap_xy = 1)."""
    import torch
    from conehead_gb300 import GridPhantom
    from conehead_gb300.phantoms import random_beam
    eng, settings = setup
    eng.prepare((64, 64, 64), (0.25, 0.25, 0.25))
    rng = np.random.default_rng(sum(size))
    rho_h = rng.uniform(0.3, 1.8, size).astype(np.float32)
    s = np.float32(0.25)
    ph = GridPhantom(rho_h, tuple(-(k - 1) * s / 2 for k in size), (s, s, s))
    rho = eng.upload_densities(ph.densities)
    src, blk = random_beam(rng, rect=(3.0, 7.0), collimator=True)
    db = eng.upload_block(blk.block_values)
    ref_job = eng.job(ph, rho, src, db, settings)
    assert ref_job.swap_xy == int(size[0] == size[1])
    ref = eng.run(ref_job).clone()
    eng.sync()
    ref = ref.cpu().numpy()
    assert ref.max() > 0
    outs = [torch.full(size, -1.0, dtype=torch.float32, device=eng.device) for _ in range(2)]
    for out in outs:                                   # two calls in a row
        call_static(eng, eng.job(ph, rho, src, db, settings, dose=out))
    eng.sync()
    for out in outs:
        assert np.abs(out.cpu().numpy() - ref).max() <= TOL * ref.max()


def test_static_refuses_grids_beyond_its_scratch(setup):
    from conehead_gb300 import _native as N
    from conehead_gb300.phantoms import random_beam, slab_phantom
    eng, settings = setup
    rng = np.random.default_rng(3)
    ph = slab_phantom(192, 0.25, seed=3, n_inserts=4)
    rho = eng.upload_densities(ph.densities)
    src, blk = random_beam(rng, field=5.0)
    db = eng.upload_block(blk.block_values)
    eng.run(eng.job(ph, rho, src, db, settings))      # prepares the plan for 192^3
    eng.sync()
    job = eng.job(ph, rho, src, db, settings)
    with pytest.raises(N.CHError) as err:
        call_static(eng, job)
    assert err.value.status == 1 and "static scratch" in str(err.value)
