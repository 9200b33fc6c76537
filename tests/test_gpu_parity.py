"""GPU parity: the CUDA path (through the C ABI) against the oracle and the
reference's own goldens.

Bars (the acceptance bars of this engine): DDA voxel sequences and the geometric intermediates
(blocked, d_eff, oad, f_soften, f_horn) bit-exact against the float32-
mirrored oracle / reference; float32 dose within 0.5% of Dmax in every
voxel above 1% of Dmax against both oracle modes (the observed maximum is
printed per case and is far below the bar); fluence / TERMA within float32
evaluation tolerance.
"""
import glob
import os
import types

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

DOSE_BAR = 5e-3          # fraction of Dmax: the 0.5% acceptance bar
DOSE_F32 = 2e-4          # observed-scale bound vs the float32-mirrored oracle


@pytest.fixture(scope="module")
def eng():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from conehead_gb300.build import build
    build()
    from conehead_gb300.conehead import engine
    return engine(0)


def dose_error(d, ref):
    """max |d - ref| / Dmax over voxels above 1% of Dmax, and over all voxels."""
    dmax = ref.max()
    mask = ref > 0.01 * dmax
    err = np.abs(d.astype(np.float64) - ref)
    return err[mask].max() / dmax, err.max() / dmax


def run_gpu(source, block, phantom, settings, intermediates=True):
    from conehead_gb300 import Conehead
    return Conehead().calculate(source, block, phantom, settings, return_intermediates=intermediates)


# ------------------------------------------------------------ geometry --
def test_cone_directions_bitexact(eng, settings, oracle_lib):
    eng.set_kernel(settings["energy_weights"])
    dirs = eng.cone_directions()
    thetas = np.arange(0, 360, 30, dtype=np.float32)
    from conehead_gb300.kernel import poly_kernel_tables
    _, _, phis = poly_kernel_tables(settings["energy_weights"])
    for i, th in enumerate(thetas):
        for j, ph in enumerate(phis):
            ref = oracle_lib.cone_direction(th, ph, oracle_lib.MODE_F32).astype(np.float32)
            assert np.array_equal(dirs[i * len(phis) + j], ref), (th, ph)


def test_dda_traces_bitexact(oracle_lib):
    from conehead_gb300.engine import dda_trace
    rng = np.random.default_rng(5)
    for trial in range(6):
        n = [int(v) for v in rng.integers(3, 60, size=3)]
        sp = rng.choice([0.1, 0.2, 0.25, 0.3, 0.5], size=3).astype(np.float32)
        k = 64
        starts = np.stack([rng.integers(0, v, size=k) for v in n], axis=1).astype(np.int32)
        d = rng.normal(size=(k, 3))
        d[rng.random(k) < 0.2, rng.integers(0, 3)] = 0.0
        d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
        vox, tv, ln = dda_trace(n, sp, starts, d, cap=256)
        for r in range(k):
            v_ref, t_ref = oracle_lib.dda(n, sp, starts[r], d[r].astype(np.float64), oracle_lib.MODE_F32)
            assert ln[r] == len(t_ref)
            L = min(ln[r], 256)
            assert np.array_equal(vox[r, :L], v_ref[:L])
            assert np.array_equal(tv[r, :L].astype(np.float64), t_ref[:L])


def test_dda_matches_dda_3d_c_where_exact(oracle_lib):
    """Against conehead's compiled Cython DDA (FP64 golden): identical voxel
    sequences whenever the float32-mirrored oracle agrees with FP64."""
    from conehead_gb300.engine import dda_trace
    g = np.load(os.path.join(GOLDEN, "dda_ref.npz"))
    off = g["offsets"]
    agree = 0
    for i in range(len(g["direction"])):
        ref = g["voxels"][off[i]:off[i + 1]]
        v32, _ = oracle_lib.dda(g["shape"][i], g["spacing"][i], g["start"][i], g["direction"][i],
                                oracle_lib.MODE_F32)
        if not np.array_equal(v32, ref):
            continue
        vox, _, ln = dda_trace(g["shape"][i], g["spacing"][i].astype(np.float32), g["start"][i][None],
                               g["direction"][i][None].astype(np.float32), cap=max(len(ref), 1))
        assert ln[0] == len(ref)
        assert np.array_equal(vox[0, :len(ref)], ref)
        agree += 1
    assert agree >= 290


# ------------------------------------------------------ golden pipelines --
PIPELINES = sorted(glob.glob(os.path.join(GOLDEN, "pipeline_*.npz")))


@pytest.mark.parametrize("path", PIPELINES, ids=[os.path.basename(p) for p in PIPELINES])
def test_reference_golden_pipeline(eng, settings, path):
    from conehead_gb300 import Block
    g = np.load(path)
    src = types.SimpleNamespace(position=g["position"], v_y=g["v_y"], transform=g["transform"],
                                sad=g["sad"][()])
    blk = Block()
    blk.set_square(float(g["square"]))
    ph = types.SimpleNamespace(size=[int(n) for n in g["size"]], origin=g["origin"], spacing=g["spacing"],
                               densities=g["densities"])
    out = run_gpu(src, blk, ph, settings)
    for k in ("blocked", "d_eff", "oad", "f_soften", "f_horn"):
        assert np.array_equal(out[k], g[k]), k
    np.testing.assert_allclose(out["fluence"], g["fluence"], rtol=2e-6, atol=1e-7 * g["fluence"].max())
    np.testing.assert_allclose(out["terma"], g["terma"], rtol=2e-5, atol=1e-6 * g["terma"].max())
    D = g["dose"].astype(np.float64)
    hot, allv = dose_error(out["dose"], D)
    print(f"{os.path.basename(path)}: max |dD|/Dmax = {hot:.2e} (>1% Dmax), {allv:.2e} (all)")
    assert allv <= 1e-4


# ------------------------------------------------------- configurations --
def compare_with_oracle(oracle_lib, source, block, phantom, settings, label, f64=True):
    out = run_gpu(source, block, phantom, settings)
    ref = oracle_lib.calculate(source, block, phantom, settings, oracle_lib.MODE_F32)
    for k in ("blocked", "d_eff", "oad", "f_soften", "f_horn"):
        assert np.array_equal(out[k].astype(np.float64), ref[k]), k
    np.testing.assert_allclose(out["terma"], ref["terma"], rtol=2e-5, atol=1e-6 * ref["terma"].max())
    hot32, all32 = dose_error(out["dose"], ref["dose"])
    msg = f"{label}: vs fp32-mirrored oracle {hot32:.2e} of Dmax"
    assert hot32 <= DOSE_F32
    if f64:
        # The reference computes in float32.  Where a blocking sub-sample lies
        # within float32 rounding of a block-map cell edge, the FP64 re-run
        # picks the neighbouring cell, so that voxel's blocked fraction (and
        # the dose of it and its neighbours) differs by one sub-sample.  The
        # GPU follows the float32 choice bit-exactly (checked above); the FP64
        # bar is held everywhere else and the flip voxels are reported.
        ref64 = oracle_lib.calculate(source, block, phantom, settings, oracle_lib.MODE_F64)
        flip = ref["blocked"] != ref64["blocked"]
        near = flip.copy()
        for ax in range(3):
            for sh in (-1, 1):
                near |= np.roll(flip, sh, axis=ax)
        D = ref64["dose"]
        hot = (D > 0.01 * D.max()) & ~near
        err64 = np.abs(out["dose"].astype(np.float64) - D)
        hot64 = err64[hot].max() / D.max()
        msg += f", vs FP64 oracle {hot64:.2e} of Dmax (all voxels {err64.max() / D.max():.2e})"
        if flip.any():
            msg += (f"; {int(flip.sum())} voxel(s) with a float32/float64 blocking flip, "
                    f"{err64[near].max() / D.max():.2e} of Dmax there")
        assert hot64 <= DOSE_BAR
    print(msg)
    return out


def test_config_water_40(eng, settings, oracle_lib):
    """Plain method, small: 40^3 water, 0.5 cm, SSD 100, 10x10 field, G=C=0."""
    from conehead_gb300 import Block, Source
    from conehead_gb300.phantoms import water_phantom
    src = Source()
    src.gantry = 0
    src.collimator = 0
    blk = Block()
    blk.set_square(10)
    compare_with_oracle(oracle_lib, src, blk, water_phantom(40, 0.5), settings, "water 40^3 10x10")


@pytest.mark.parametrize("seed", [1, 2])
def test_config_hetero_oblique(eng, settings, oracle_lib, seed):
    from conehead_gb300.phantoms import random_beam, slab_phantom
    rng = np.random.default_rng(seed)
    ph = slab_phantom(48, 0.5, seed=seed, n_inserts=6)
    src, blk = random_beam(rng, rect=(2.0, 12.0), collimator=True)
    compare_with_oracle(oracle_lib, src, blk, ph, settings, f"hetero 48^3 seed {seed}")


def test_config_hetero_128_full_size(eng, settings, oracle_lib):
    """Plain method, heterogeneous: 128^3 at 0.25 cm, 5x5 field, random gantry."""
    from conehead_gb300.phantoms import random_beam, slab_phantom
    rng = np.random.default_rng(11)
    src, blk = random_beam(rng, field=5.0)
    compare_with_oracle(oracle_lib, src, blk, slab_phantom(128, 0.25, seed=11), settings,
                        "hetero 128^3 5x5", f64=True)


def test_config_large_field_96(eng, settings, oracle_lib):
    """A large oblique field: 96^3 heterogeneous phantom at 0.25 cm, 15 x 12 cm
    jaws, gantry 217, collimator 63."""
    from conehead_gb300 import Block, Source
    from conehead_gb300.phantoms import slab_phantom
    src = Source()
    src.gantry = 217.0
    src.collimator = 63.0
    blk = Block()
    blk.set_rect(-7.5, 7.5, -6.0, 6.0)
    compare_with_oracle(oracle_lib, src, blk, slab_phantom(96, 0.25, seed=96), settings,
                        "hetero 96^3 15x12 oblique", f64=True)


# ------------------------------------------------------------ paths agree --
@pytest.mark.parametrize("method", [0, 1], ids=["spectral", "gather"])
def test_large_ragged_grid_cone_equals_scatter(eng, settings, method):
    """250 x 224 x 163 voxels at 0.2 cm (50 x 45 x 33 cm): walks of up to
    ~640 taps, FFT periods of 512 on every axis (spectral), ragged tiles on
    every axis (gather), a field larger than one tile.  Both cone methods
    must equal the plain per-voxel scatter, whose indexing is the
    reference's loop."""
    from conehead_gb300 import GridPhantom
    from conehead_gb300.phantoms import random_beam
    rng = np.random.default_rng(250)
    n = (250, 224, 163)
    rho = np.ones(n, dtype=np.float32)
    rho[:, 60:110, :] = 0.3
    rho[100:150, 120:140, 40:90] = 1.8
    s = np.float32(0.2)
    ph = GridPhantom(rho, tuple(-(k - 1) * s / 2 for k in n), (s, s, s))
    src, blk = random_beam(rng, rect=(6.0, 10.0), collimator=True)
    eng.set_kernel(settings["energy_weights"])
    eng.set_tuning(cone_method=method)
    try:
        r = eng.upload_densities(ph.densities)
        db = eng.block_for(blk)
        a = eng.run(eng.job(ph, r, src, db, settings)).clone()
        b = eng.run(eng.job(ph, r, src, db, settings), scatter=True)
        eng.sync()
    finally:
        eng.set_tuning()
    a, b = a.cpu().numpy(), b.cpu().numpy()
    assert b.max() > 0
    err = np.abs(a - b).max() / b.max()
    print(f"250x224x163 {('spectral', 'gather')[method]} vs scatter: {err:.2e} of Dmax")
    assert err <= 2e-5


@pytest.mark.parametrize("method", [0, 1], ids=["spectral", "gather"])
def test_cone_equals_scatter(eng, settings, method):
    from conehead_gb300.phantoms import random_beam, slab_phantom
    rng = np.random.default_rng(3)
    ph = slab_phantom(64, 0.25, seed=3)
    src, blk = random_beam(rng, field=6.0)
    eng.set_kernel(settings["energy_weights"])
    eng.set_tuning(cone_method=method)
    try:
        rho = eng.upload_densities(ph.densities)
        db = eng.upload_block(blk.block_values)
        a = eng.run(eng.job(ph, rho, src, db, settings)).clone()
        b = eng.run(eng.job(ph, rho, src, db, settings), scatter=True)
        eng.sync()
    finally:
        eng.set_tuning()
    a, b = a.cpu().numpy(), b.cpu().numpy()
    assert np.abs(a - b).max() <= 2e-5 * b.max()


def test_batch_equals_single(eng, settings):
    from conehead_gb300.phantoms import random_beam, slab_phantom
    rng = np.random.default_rng(4)
    phs = [slab_phantom(n, 0.25, seed=n) for n in (40, 64, 52)]
    eng.set_kernel(settings["energy_weights"])
    jobs, singles = [], []
    for i in range(5):
        ph = phs[i % 3]
        src, blk = random_beam(rng, rect=(2.0, 10.0), collimator=True)
        rho = eng.upload_densities(ph.densities)
        db = eng.upload_block(blk.block_values)
        singles.append(eng.run(eng.job(ph, rho, src, db, settings)).clone())
        eng.sync()
        jobs.append(eng.job(ph, rho, src, db, settings))
    batch = eng.run_batch(jobs)
    eng.sync()
    for s, b in zip(singles, batch):
        s, b = s.cpu().numpy(), b.cpu().numpy()
        assert np.abs(s - b).max() <= 1e-5 * max(s.max(), 1e-30)


# ------------------------------------------------------------ edge cases --
def test_closed_jaws_give_zero_dose(eng, settings):
    from conehead_gb300 import Block, Source
    from conehead_gb300.phantoms import water_phantom
    src = Source()
    src.gantry = 10.0
    out = run_gpu(src, Block(), water_phantom(20, 0.5), settings)
    assert not out["dose"].any() and not out["terma"].any()


def test_beam_missing_the_grid(eng, settings):
    from conehead_gb300 import Block, GridPhantom, Source
    src = Source()
    src.gantry = 0
    blk = Block()
    blk.set_rect(-2.0, 2.0, -2.0, 2.0)
    ph = GridPhantom(np.ones((16, 16, 16), np.float32), (30.0, 0.0, 30.0), (0.5, 0.5, 0.5))
    out = run_gpu(src, blk, ph, settings)
    assert not out["dose"].any()


@pytest.mark.parametrize("size,spacing,samples", [
    ((1, 1, 1), (0.5, 0.5, 0.5), 3),
    ((2, 3, 5), (0.4, 0.5, 0.3), 3),
    ((21, 21, 37), (0.5, 0.5, 0.5), 1),
    ((24, 24, 17), (0.3, 0.3, 0.6), 2),
    ((12, 12, 12), (0.5, 0.5, 0.5), 4),
])
def test_ragged_grids_and_resampling(eng, settings, oracle_lib, size, spacing, samples):
    from conehead_gb300 import Block, GridPhantom, Source
    rng = np.random.default_rng(sum(size))
    rho = rng.uniform(0.3, 1.8, size).astype(np.float32)
    origin = [-(n - 1) * s / 2 for n, s in zip(size, spacing)]
    ph = GridPhantom(rho, origin, spacing)
    src = Source()
    src.gantry = 25.0
    src.collimator = 10.0
    blk = Block()
    blk.set_rect(-3.0, 2.0, -2.5, 3.5)
    st = dict(settings)
    st["fluenceResampling"] = samples
    out = run_gpu(src, blk, ph, st)
    ref = oracle_lib.calculate(src, blk, ph, st, oracle_lib.MODE_F32)
    for k in ("blocked", "d_eff", "oad"):
        assert np.array_equal(out[k].astype(np.float64), ref[k]), k
    if ref["dose"].max() > 0:
        assert np.abs(out["dose"] - ref["dose"]).max() <= DOSE_F32 * ref["dose"].max()


def test_fresh_source_float32_geometry(eng, settings, oracle_lib):
    from conehead_gb300 import Block, Source
    from conehead_gb300.phantoms import slab_phantom
    src = Source()                       # angles never set: float32 arrays
    assert src.position.dtype == np.float32
    blk = Block()
    blk.set_square(6.0)
    compare_with_oracle(oracle_lib, src, blk, slab_phantom(32, 0.5, seed=9, n_inserts=4), settings,
                        "fresh source 32^3", f64=False)


def test_mlc_like_transmission_values(eng, settings, oracle_lib):
    """Fractional transmission (MLC leaf edges) takes the general blocked sum."""
    from conehead_gb300 import Block, Source
    from conehead_gb300.phantoms import slab_phantom
    src = Source()
    src.gantry = 300.0
    blk = Block()
    blk.set_rect(-4.0, 4.0, -4.0, 4.0)
    blk.block_values[1600:1700, 1600:2400] = 0.25
    blk.block_values[2200:2210, :] *= 0.5
    compare_with_oracle(oracle_lib, src, blk, slab_phantom(40, 0.5, seed=2, n_inserts=5), settings,
                        "mlc-like 40^3", f64=False)


def test_parallel_ray_raises(eng, settings):
    from conehead_gb300 import Block, GridPhantom, Source
    src = Source()
    src.gantry = 0
    blk = Block()
    blk.set_square(10)
    # the row y = -100 holds voxels in the source's own plane: n . (S - p) = 0
    ph = GridPhantom(np.ones((4, 4, 4), np.float32), (-1.0, -101.0, -1.0), (1.0, 1.0, 1.0))
    with pytest.raises(RuntimeError, match="plane"):
        run_gpu(src, blk, ph, settings)


def test_dose_is_linear_in_source_strength(eng, settings):
    from conehead_gb300.phantoms import random_beam, slab_phantom
    rng = np.random.default_rng(8)
    ph = slab_phantom(40, 0.5, seed=8, n_inserts=4)
    src, blk = random_beam(rng, field=8.0)
    a = run_gpu(src, blk, ph, settings, intermediates=False)
    st = dict(settings)
    for k in ("sPri", "sAnn", "sExp"):
        st[k] = settings[k] * 2.0
    b = run_gpu(src, blk, ph, st, intermediates=False)
    assert np.abs(b - 2.0 * a).max() <= 1e-5 * b.max()
