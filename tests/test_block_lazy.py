"""Jaw blocks without a host map.

``Block.set_square`` / ``set_rect`` only record their openings until
``block_values`` is read; the engine then sends the opening to the GPU as a
uniform crop (no memory).  These CPU tests check that the recorded opening is
exactly the nonzero box of the map the reference's code would paint
(conehead/block.py:64-85, numpy slice rules included), and that blocks whose
map is not one rectangle of ones, or whose map was read, take the map path.
"""
import numpy as np


def _map_box(values):
    from conehead_gb300 import _native as N
    crop, r0, c0 = N.block_crop(values)
    if not values.any():
        return (0, 0, 0, 0), True
    return (r0, r0 + crop.shape[0], c0, c0 + crop.shape[1]), bool(np.all(crop == 1))


def test_rect_equals_painted_map():
    from conehead_gb300.block import Block
    rng = np.random.default_rng(12)
    sizes = [0.0, 0.01, 0.3, 1.0, 2.5, 5.0, 10.0, 12.3, 39.99, 40.0, 45.0, 50.0, 79.0]
    for L in sizes + list(rng.uniform(0, 60, 30)):
        b = Block()
        b.set_square(L)
        rect = b.device_rect()
        box, ones = _map_box(b.block_values)
        assert ones and rect == box, L
    for _ in range(40):
        x = np.sort(rng.uniform(-25, 25, 2))
        z = np.sort(rng.uniform(-25, 25, 2))
        b = Block()
        b.set_rect(x[0], x[1], z[0], z[1])
        rect = b.device_rect()
        box, ones = _map_box(b.block_values)
        assert ones and rect == box


def test_nested_openings_are_one_rectangle_and_others_are_not():
    from conehead_gb300.block import Block
    b = Block()
    b.set_rect(-3, 4, -2, 5)
    b.set_square(2)
    rect = b.device_rect()
    box, ones = _map_box(b.block_values)
    assert ones and rect == box
    b = Block()
    b.set_rect(-3, 4, -2, 5)
    b.set_rect(5, 6, -1, 1)
    assert b.device_rect() is None           # an L-shaped opening: the engine uploads the map


def test_reading_or_editing_the_map_switches_to_the_map():
    from conehead_gb300.block import Block
    b = Block()
    b.set_square(5)
    assert b.device_rect() == (1750, 2250, 1750, 2250)
    v = b.block_values
    v[2000, 2000] = 0.5                      # caller edits the map in place
    assert b.device_rect() is None
    b.set_square(10)                         # later openings paint into the map
    assert b.block_values[1600, 1600] == 1 and b.block_values[2000, 2000] == 1
    c = Block()
    c.block_values = np.ones((4000, 4000), dtype=np.float32)
    assert c.device_rect() is None and c.device_mlc() is None


def test_transmission_reads_the_lazy_map():
    from conehead_gb300.block import Block
    b = Block()
    b.set_square(10)
    assert b.transmission(np.array([0.0, 0.0], dtype=np.float32)) == 1
    assert b.transmission(np.array([6.0, 0.0], dtype=np.float32)) == 0
