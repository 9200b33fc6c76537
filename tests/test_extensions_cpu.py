"""The physics extensions (not in the reference) on the CPU oracle, and
their settings keys.

* Radiological cone distance with unit density is the geometric walk, so the
  extended cone equals the reference cone exactly in water.
* Cones in the beam frame with the identity orientation are the room-frame
  cones exactly.
* Both change the dose where they should: in a lung slab, and for a turned
  beam.
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def tables(settings):
    from conehead_gb300.kernel import poly_kernel_tables
    return poly_kernel_tables(settings["energy_weights"])


def test_settings_keys_to_option_bits(settings):
    from conehead_gb300 import _native as N
    assert N.physics_options(settings) == 0
    assert N.physics_options(dict(settings, coneDistance="radiological")) == N.CH_OPT_RADIOLOGICAL_DISTANCE
    assert N.physics_options(dict(settings, coneFrame="beam")) == N.CH_OPT_CONES_IN_BEAM_FRAME
    assert N.physics_options(dict(settings, coneFrame="beam", coneDistance="radiological")) == 3
    with pytest.raises(ValueError):
        N.physics_options(dict(settings, coneFrame="gantry"))
    assert N.settings_struct(dict(settings, coneFrame="beam")).options == 2


def test_extensions_reduce_to_the_reference(oracle_lib, tables):
    K, th, ph = tables
    size = [10, 12, 9]
    rng = np.random.default_rng(3)
    T = rng.random(size) * (rng.random(size) > 0.85)
    ref = oracle_lib.cone(T, size, [0.5] * 3, K, th, ph, oracle_lib.MODE_F32)
    water = oracle_lib.cone_ext(T, size, [0.5] * 3, K, th, ph, oracle_lib.MODE_F32,
                                rho=np.ones(size, np.float32))
    assert np.array_equal(water, ref)
    ident = oracle_lib.cone_ext(T, size, [0.5] * 3, K, th, ph, oracle_lib.MODE_F32, frame=np.eye(3))
    assert np.array_equal(ident, ref)
    # lung (rho 0.25): the kernel reaches further, so less energy stays near the source
    lung = oracle_lib.cone_ext(T, size, [0.5] * 3, K, th, ph, oracle_lib.MODE_F32,
                               rho=np.full(size, 0.25, np.float32))
    assert np.abs(lung - ref).max() > 1e-2 * ref.max()
    # a turned frame moves dose around but keeps the total deposited inside a big grid
    c, s_ = np.cos(0.7), np.sin(0.7)
    rot = np.array([[c, -s_, 0], [s_, c, 0], [0, 0, 1.0]])
    turned = oracle_lib.cone_ext(T, size, [0.5] * 3, K, th, ph, oracle_lib.MODE_F32, frame=rot)
    assert np.abs(turned - ref).max() > 1e-3 * ref.max()
