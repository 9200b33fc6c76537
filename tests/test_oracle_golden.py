"""Pin the CPU oracle to the reference before trusting it.

* DDA: the oracle's FP64 trace equals conehead's compiled Cython dda_3d_c
  (tests/golden/dda_ref.npz) voxel for voxel and t-value for t-value.
* Whole path: the oracle's float32-mirrored mode equals the reference's own
  Conehead.calculate() run under the Numba-typed stand-in
  (tests/golden/pipeline_*.npz): blocked, d_eff, oad, fluence, f_soften and
  f_horn bit-exact; TERMA within 1e-6 relative (float32 exp rounding) and
  dose within 2e-5 of Dmax (float32 atomic summation order).
* FP32-mirrored vs FP64 modes agree to 0.5% of Dmax (the engine's bar).
"""
import glob
import os
import types

import numpy as np
import pytest

from conftest import GOLDEN
from conehead_gb300 import Block, GridPhantom, Source

PIPELINES = sorted(glob.glob(os.path.join(GOLDEN, "pipeline_*.npz")))


def test_dda_fp64_matches_dda_3d_c(oracle_lib):
    g = np.load(os.path.join(GOLDEN, "dda_ref.npz"))
    off = g["offsets"]
    assert len(g["direction"]) >= 300
    for i in range(len(g["direction"])):
        v, t = oracle_lib.dda(g["shape"][i], g["spacing"][i], g["start"][i],
                              g["direction"][i], oracle_lib.MODE_F64)
        assert np.array_equal(v, g["voxels"][off[i]:off[i + 1]]), i
        assert np.array_equal(t, g["tvals"][off[i]:off[i + 1]]), i


def test_dda_notebook_known_answer(oracle_lib):
    # dda_benchmarking.ipynb: dir (1,2,3)/sqrt(14) from (50,50,50) in 101^3 unit voxels
    d = np.array([1, 2, 3]) / np.sqrt(14)
    v, t = oracle_lib.dda((101, 101, 101), (1, 1, 1), (50, 50, 50), d, oracle_lib.MODE_F64)
    np.testing.assert_allclose(t[:4], [0.5 * np.sqrt(14) / 3, 0.5 * np.sqrt(14) / 2,
                                       1.5 * np.sqrt(14) / 3, 0.5 * np.sqrt(14)], rtol=1e-12)
    assert tuple(v[0]) == (50, 50, 50) and tuple(v[1]) == (50, 50, 51)


def _case(path):
    g = np.load(path)
    src = types.SimpleNamespace(position=g["position"], v_y=g["v_y"],
                                transform=g["transform"], sad=g["sad"][()])
    block = Block()
    block.set_square(float(g["square"]))
    ph = types.SimpleNamespace(size=[int(n) for n in g["size"]], origin=g["origin"],
                               spacing=g["spacing"], densities=g["densities"])
    return g, src, block, ph


@pytest.mark.parametrize("path", PIPELINES, ids=[os.path.basename(p) for p in PIPELINES])
def test_oracle_matches_reference_calculate(oracle_lib, settings, path):
    g, src, block, ph = _case(path)
    out = oracle_lib.calculate(src, block, ph, settings, oracle_lib.MODE_F32)
    assert (g["terma"] > 0).sum() > 100
    for k in ("blocked", "d_eff", "oad", "fluence", "f_soften", "f_horn"):
        assert np.array_equal(out[k], g[k].astype(np.float64)), k
    T = g["terma"].astype(np.float64)
    np.testing.assert_allclose(out["terma"], T, rtol=1e-6, atol=1e-6 * T.max())
    D = g["dose"].astype(np.float64)
    assert np.abs(out["dose"] - D).max() <= 2e-5 * D.max()


def test_fp32_vs_fp64_small_field(oracle_lib, settings):
    s = Source()
    s.gantry = 20.0
    b = Block()
    b.set_rect(-2.0, 3.0, -1.5, 2.5)
    rng = np.random.default_rng(3)
    rho = rng.uniform(0.3, 1.8, (18, 18, 18)).astype(np.float32)
    ph = GridPhantom(rho, (-4.25, -4.25, -4.25), (0.5, 0.5, 0.5))
    a = oracle_lib.calculate(s, b, ph, settings, oracle_lib.MODE_F32)["dose"]
    c = oracle_lib.calculate(s, b, ph, settings, oracle_lib.MODE_F64)["dose"]
    assert c.max() > 0
    assert np.abs(a - c).max() <= 5e-3 * c.max()
