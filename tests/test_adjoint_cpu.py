"""The facts the beamlet adjoint rests on, checked on the CPU oracle.

* The oracle's transposed cone is the transpose of its cone (the reference
  scatter, conehead/conehead.py:385-488): <C^T r, t> = <r, C t> in float64.
* The blocked fraction is linear in the block-map values, and TERMA is
  quadratic in them: blocked(a w) = a blocked(w) and T(a w) = a^2 T(w)
  (fluence and TERMA each carry one factor of blocked,
  conehead/conehead.py:641-662), which gives dT/dblocked = 2 T / blocked.
* The beamlet grid geometry and its host block map.
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def tables(settings):
    from conehead_gb300.kernel import poly_kernel_tables
    return poly_kernel_tables(settings["energy_weights"])


def test_oracle_transpose_identity(oracle_lib, tables):
    K, th, ph = tables
    rng = np.random.default_rng(1)
    size = [9, 11, 8]
    r = rng.random(size)
    t = rng.random(size) * (rng.random(size) > 0.8)
    ct = oracle_lib.cone(t, size, [0.5] * 3, K, th, ph, oracle_lib.MODE_F64)
    ctr = oracle_lib.cone_transpose(r, size, [0.5] * 3, K, th, ph, oracle_lib.MODE_F64)
    lhs, rhs = float((ctr * t).sum()), float((r * ct).sum())
    assert abs(lhs - rhs) <= 1e-12 * abs(rhs)
    # a point response: C^T of a unit impulse at v is the set of walk weights reaching v
    e = np.zeros(size)
    e[4, 5, 3] = 1.0
    col = oracle_lib.cone_transpose(e, size, [0.5] * 3, K, th, ph, oracle_lib.MODE_F64)
    for s in [(4, 5, 3), (2, 7, 1), (8, 0, 6)]:
        u = np.zeros(size)
        u[s] = 1.0
        row = oracle_lib.cone(u, size, [0.5] * 3, K, th, ph, oracle_lib.MODE_F64)
        assert row[4, 5, 3] == pytest.approx(col[s], rel=1e-14, abs=1e-300)


def test_terma_is_quadratic_in_the_block_map(oracle_lib, settings):
    from conehead_gb300 import Source
    from conehead_gb300.adjoint import BeamletGrid, MapBlock
    from conehead_gb300.phantoms import slab_phantom
    ph = slab_phantom(20, 0.5, seed=4, n_inserts=3)
    src = Source()
    src.gantry = 15.0
    src.collimator = 0.0
    bl = BeamletGrid.square(6, 1.0)
    w = np.random.default_rng(2).uniform(0.1, 1.0, bl.shape).astype(np.float32)
    a = np.float32(2.0)                       # exact in float32: the scaled map is exact
    p1 = oracle_lib.prologue(src, MapBlock(bl.host_map(w)), ph, settings, oracle_lib.MODE_F64)
    p2 = oracle_lib.prologue(src, MapBlock(bl.host_map(a * w)), ph, settings, oracle_lib.MODE_F64)
    assert p1["blocked"].max() > 0
    np.testing.assert_allclose(p2["blocked"], 2.0 * p1["blocked"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(p2["terma"], 4.0 * p1["terma"], rtol=1e-12, atol=0)
    # blocked is linear: two disjoint halves of the map add up
    w_lo, w_hi = w.copy(), w.copy()
    w_lo[:3] = 0
    w_hi[3:] = 0
    b_lo = oracle_lib.prologue(src, MapBlock(bl.host_map(w_lo)), ph, settings, oracle_lib.MODE_F64)["blocked"]
    b_hi = oracle_lib.prologue(src, MapBlock(bl.host_map(w_hi)), ph, settings, oracle_lib.MODE_F64)["blocked"]
    np.testing.assert_allclose(b_lo + b_hi, p1["blocked"], rtol=1e-13, atol=1e-15)


def test_beamlet_grid_geometry():
    from conehead_gb300.adjoint import BeamletGrid
    bl = BeamletGrid.square(40, 0.5)
    assert (bl.rows, bl.cols, bl.cell_rows, bl.cell_cols, bl.r0, bl.c0) == (40, 40, 50, 50, 1000, 1000)
    assert bl.crop_shape == (2000, 2000)
    w = np.arange(1600, dtype=np.float32).reshape(40, 40)
    m = bl.host_map(w)
    assert m.shape == (4000, 4000) and m[999, 1500] == 0 and m[1000, 1000] == 0 and m[1049, 1049] == 0
    assert m[1050, 1000] == 40 and m[2999, 2999] == 1599 and m[3000, 2999] == 0
    s = bl.struct()
    assert (s.rows, s.cols, s.cell_rows, s.cell_cols, s.r0, s.c0) == (40, 40, 50, 50, 1000, 1000)
    with pytest.raises(ValueError):
        BeamletGrid.square(90, 0.5)           # 45 cm does not fit the 40 cm map


def test_fp64_chain_rule_gradient_equals_oracle_differences(oracle_lib, settings):
    """The FP64 beamlet gradient by the chain rule (forward, C^T on the TERMA
    support, dTERMA/dblocked = 2 T / blocked, transposed blocking onto the
    beamlets) equals central differences of the FP64 oracle's own objective.
    This pins the checker that the full-size GPU gradient is compared with."""
    from conehead_gb300 import Source
    from conehead_gb300.adjoint import BeamletGrid, MapBlock, sphere_target
    from conehead_gb300.phantoms import slab_phantom
    ph = slab_phantom(20, 0.5, seed=6, n_inserts=3)
    src = Source()
    src.gantry = 35.0
    src.collimator = 0.0
    bl = BeamletGrid.square(6, 1.0)
    rng = np.random.default_rng(12)
    w = rng.uniform(0.0, 1.0, bl.shape).astype(np.float32)
    target = sphere_target(ph, (0.5, 0.0, -0.5), 2.0)
    grad, dose = oracle_lib.beamlet_gradient_f64(src, bl, w, ph, settings, target)
    assert dose.max() > 0 and np.abs(grad).max() > 0

    def loss(weights):
        d = oracle_lib.calculate(src, MapBlock(bl.host_map(weights)), ph, settings, oracle_lib.MODE_F64)["dose"]
        return float(((d - target) ** 2).sum())

    h = 1e-4
    flat = [(i, j) for i in range(bl.rows) for j in range(bl.cols)]
    picks = [flat[k] for k in rng.choice(len(flat), 8, replace=False)]
    for i, j in picks:
        wp, wm = w.copy(), w.copy()
        wp[i, j] = np.float32(w[i, j] + h)
        wm[i, j] = np.float32(w[i, j] - h)
        fd = (loss(wp) - loss(wm)) / (float(wp[i, j]) - float(wm[i, j]))
        # L is quartic in w (the dose is quadratic), so the central difference
        # is off by O(h^2) terms, far below this bound
        assert abs(grad[i, j] - fd) <= 1e-6 * np.abs(grad).max(), (i, j, grad[i, j], fd)
