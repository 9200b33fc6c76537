"""GPU: the spectral cone stage (the default cone method).

* Doses of the spectral method and the stencil gather agree on mixed grid
  shapes, non-cubic grids with anisotropic voxels, odd beam counts (the last
  pair of a launch holds one beam) and batches of more than 32 beams (more
  than one launch per grid shape, reusing one work arena).
* Axes of 97-128 voxels (period 256, the passes with one butterfly per thread
  and stage) agree with the gather on every axis and on odd sizes; so do
  axes at periods 384, 192 and 128 (the 16 x N2 kernels), mixed per grid.
* The cone operator C and its transpose agree between the two methods on a
  random sparse input, also with two axes at period 256 and with the 16 x N2
  kernels on every axis (50 x 150 x 66: periods 128, 384, 192).
* The stencil spectrum of a grid shape is built by ch_plan_prepare, counted
  in ch_plan_memory's tables, reused by the next call and dropped when the
  kernel changes.
* An unknown cone method is refused.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 2e-6     # fraction of the larger dose: both methods are float32


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
    yield e
    e.close()


def _doses(eng, jobs, method):
    eng.set_tuning(cone_method=method)
    try:
        eng.run_batch(jobs)
        eng.sync()
        return [j.dose.cpu().numpy().copy() for j in jobs]
    finally:
        eng.set_tuning()


def _grid_phantom(n, spacing, seed):
    from conehead_gb300 import GridPhantom
    rng = np.random.default_rng(seed)
    rho = np.ones(n, dtype=np.float32)
    rho[:, : n[1] // 3, :] = 0.3
    for _ in range(4):
        lo = [int(rng.integers(0, k - 4)) for k in n]
        hi = [lo[k] + int(rng.integers(2, max(3, n[k] // 3))) for k in range(3)]
        rho[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] = rng.uniform(0.2, 2.0)
    sp = tuple(np.float32(x) for x in spacing)
    return GridPhantom(rho, tuple(-(k - 1) * s / 2 for k, s in zip(n, sp)), sp)


def test_spectral_equals_gather_mixed_batch(eng, settings):
    from conehead_gb300.phantoms import random_beam, slab_phantom
    rng = np.random.default_rng(71)
    phs = [slab_phantom(48, 0.25, seed=1, n_inserts=5), _grid_phantom((37, 50, 29), (0.25, 0.25, 0.25), 2),
           _grid_phantom((61, 40, 45), (0.25, 0.25, 0.25), 3)]
    rhos = [eng.upload_densities(p.densities) for p in phs]
    jobs = []
    for i in range(7):                                  # 3 + 2 + 2 beams: odd counts per shape
        k = i % 3
        src, blk = random_beam(rng, rect=(2.0, 9.0), collimator=True)
        jobs.append(eng.job(phs[k], rhos[k], src, eng.block_for(blk), settings))
    spec = _doses(eng, jobs, 0)
    gath = _doses(eng, jobs, 1)
    worst = 0.0
    for a, b in zip(spec, gath):
        assert b.max() > 0
        worst = max(worst, np.abs(a - b).max() / b.max())
    print(f"spectral vs gather, 7 beams on 48^3 / 37x50x29 / 61x40x45: {worst:.2e} of Dmax")
    assert worst <= TOL


def test_spectral_anisotropic_voxels_and_many_beams(eng, settings):
    from conehead_gb300.phantoms import random_beam
    rng = np.random.default_rng(72)
    ph = _grid_phantom((40, 33, 52), (0.3, 0.25, 0.2), 4)
    rho = eng.upload_densities(ph.densities)
    jobs = []
    for _ in range(35):                                 # 18 pairs: two launches of at most 16 pairs
        src, blk = random_beam(rng, rect=(2.0, 8.0), collimator=True)
        jobs.append(eng.job(ph, rho, src, eng.block_for(blk), settings))
    spec = _doses(eng, jobs, 0)
    gath = _doses(eng, jobs, 1)
    worst = max(np.abs(a - b).max() / b.max() for a, b in zip(spec, gath))
    print(f"spectral vs gather, 35 beams on 40x33x52 at 0.3/0.25/0.2 cm: {worst:.2e} of Dmax")
    assert worst <= TOL


def test_spectral_period_256_axes(eng, settings):
    """Axes of 97-128 voxels take period 256, whose passes run the two radix-16
    stages with one butterfly per thread and global loads and stores from the
    stages themselves: all three axes at 256 with a line count that is not a
    multiple of 16 (99 x 101), and x at the largest size for the period with
    z odd at the smallest (128 x 36 x 97)."""
    from conehead_gb300.phantoms import random_beam
    rng = np.random.default_rng(73)
    sp = (0.3, 0.3, 0.25)                               # one spacing per call
    phs = [_grid_phantom((99, 101, 120), sp, 5), _grid_phantom((128, 36, 97), sp, 6)]
    rhos = [eng.upload_densities(p.densities) for p in phs]
    jobs = []
    for i in range(5):                                  # 3 + 2 beams: the last pair of the first shape holds one
        k = i % 2
        src, blk = random_beam(rng, rect=(2.0, 9.0), collimator=True)
        jobs.append(eng.job(phs[k], rhos[k], src, eng.block_for(blk), settings))
    spec = _doses(eng, jobs, 0)
    gath = _doses(eng, jobs, 1)
    worst = 0.0
    for a, b in zip(spec, gath):
        assert b.max() > 0
        worst = max(worst, np.abs(a - b).max() / b.max())
    print(f"spectral vs gather, 5 beams on 99x101x120 / 128x36x97: {worst:.2e} of Dmax")
    assert worst <= TOL


def test_spectral_16xn2_periods_per_axis(eng, settings):
    """Axes at FFT periods 384, 192 and 128 take the 16 x N2 pass kernels
    (N2 = 24, 12, 8), chosen per axis: 150 x 70 x 50 (x at 384, y at 192,
    z at 128) and 66 x 180 x 90 (x at 192, y at 384, z at 192), three beams
    each (the last pair of a shape holds one), against the gather."""
    from conehead_gb300.phantoms import random_beam
    rng = np.random.default_rng(74)
    sp = (0.25, 0.25, 0.25)
    phs = [_grid_phantom((150, 70, 50), sp, 7), _grid_phantom((66, 180, 90), sp, 8)]
    rhos = [eng.upload_densities(p.densities) for p in phs]
    jobs = []
    for i in range(6):
        k = i % 2
        src, blk = random_beam(rng, rect=(2.0, 8.0), collimator=True)
        jobs.append(eng.job(phs[k], rhos[k], src, eng.block_for(blk), settings))
    spec = _doses(eng, jobs, 0)
    gath = _doses(eng, jobs, 1)
    worst = 0.0
    for a, b in zip(spec, gath):
        assert b.max() > 0
        worst = max(worst, np.abs(a - b).max() / b.max())
    print(f"spectral vs gather, 6 beams on 150x70x50 / 66x180x90: {worst:.2e} of Dmax")
    assert worst <= TOL


@pytest.mark.parametrize("size", [(29, 36, 31), (100, 36, 110), (50, 150, 66)])
def test_spectral_operator_and_transpose(eng, settings, size):
    import torch
    from conehead_gb300.adjoint import cone
    spacing = (0.4, 0.4, 0.4)
    g = torch.Generator().manual_seed(5)
    x = torch.rand(size, generator=g) * (torch.rand(size, generator=g) > 0.9)
    x = x.cuda()
    out = {}
    for method in (0, 1):
        eng.set_tuning(cone_method=method)
        try:
            out[method] = [cone(eng, size, spacing, x, transpose=t).cpu().numpy() for t in (False, True)]
        finally:
            eng.set_tuning()
    for t in range(2):
        a, b = out[0][t], out[1][t]
        err = np.abs(a - b).max() / np.abs(b).max()
        print(f"{'C^T' if t else 'C'} spectral vs gather, {size}: {err:.2e} of max")
        assert err <= TOL


def test_spectrum_cache_follows_prepare_and_kernel(eng, settings):
    from conehead_gb300 import _native as N

    def tables():
        t, s = ctypes.c_size_t(), ctypes.c_size_t()
        N.check(eng.L.ch_plan_memory(eng.plan, ctypes.byref(t), ctypes.byref(s)), "ch_plan_memory")
        return t.value

    spectrum = 48 * 48 * 48 * 8                          # periods of 24 x 20 x 18: 48 (3 x 16) each, complex float32
    eng.set_kernel(settings["energy_weights"])
    eng.prepare((32, 32, 32), (0.5, 0.5, 0.5))          # stencils for this spacing (and 32^3's spectrum)
    before = tables()
    eng.prepare((24, 20, 18), (0.5, 0.5, 0.5))
    built = tables()
    assert built - before == spectrum                    # only the new shape's spectrum
    eng.prepare((24, 20, 18), (0.5, 0.5, 0.5))
    assert tables() == built                             # built once per shape
    w2 = dict(settings["energy_weights"])
    w2["1.0"] = w2["1.0"] * 1.5
    try:
        eng.set_kernel(w2)                               # new tap weights: every spectrum is dropped
        assert tables() <= built - spectrum
    finally:
        eng.set_kernel(settings["energy_weights"])


def test_unknown_cone_method_is_refused(eng):
    from conehead_gb300 import _native as N
    with pytest.raises(N.CHError, match="cone_method"):
        eng.set_tuning(cone_method=7)
    eng.set_tuning()
