"""Seeded synthetic phantoms and beams for the benchmark workloads.

No dataset is involved: every input is generated from
``numpy.random.default_rng(seed)``.

* ``water_phantom`` -- homogeneous water box, surface on the isocentre
  plane (the conehead SimplePhantom convention, SSD = SAD = 100 cm).
* ``slab_phantom`` -- heterogeneous box centred on the isocentre: water
  (1.0), a lung slab (0.25) at depth 5-12 cm and a bone slab (1.85) at
  depth 14-16 cm below the y = min surface, plus ``n_inserts`` random
  cuboids with density uniform in [0.2, 2.0].
* ``random_beam`` -- gantry (and optionally collimator) angle and a square
  or rectangular jaw field drawn from the generator.
"""
import numpy as np

from .block import Block
from .phantom import GridPhantom
from .source import Source


def water_phantom(n=40, spacing=0.5, density=1.0):
    """n^3 water box, x/z centred on the beam axis, surface at y = 0."""
    s = np.float32(spacing)
    origin = (-(n - 1) * s / 2, s / 2, -(n - 1) * s / 2)
    return GridPhantom(np.full((n, n, n), density, dtype=np.float32), origin, (s, s, s))


def slab_phantom(n=128, spacing=0.25, seed=0, n_inserts=20):
    s = float(np.float32(spacing))
    rng = np.random.default_rng(seed)
    rho = np.ones((n, n, n), dtype=np.float32)
    depth = (np.arange(n) + 0.5) * s          # depth of voxel centres below the y-min face
    lung = (depth >= 5.0) & (depth < 12.0)
    bone = (depth >= 14.0) & (depth < 16.0)
    rho[:, lung, :] = 0.25
    rho[:, bone, :] = 1.85
    for _ in range(n_inserts):
        size = rng.integers(max(2, n // 32), max(3, n // 6), size=3)
        lo = [int(rng.integers(0, n - int(sz))) for sz in size]
        val = np.float32(rng.uniform(0.2, 2.0))
        rho[lo[0]:lo[0] + size[0], lo[1]:lo[1] + size[1], lo[2]:lo[2] + size[2]] = val
    origin = (-(n - 1) * s / 2,) * 3
    return GridPhantom(rho, origin, (s, s, s))


def random_beam(rng, field=5.0, rect=None, collimator=False):
    """(Source, Block): gantry ~ U[0, 360), square field or jaw rectangle.

    ``rect`` = (lo, hi) draws jaw X and Y sizes uniformly in [lo, hi] cm.
    """
    src = Source()
    src.gantry = float(rng.uniform(0.0, 360.0))
    if collimator:
        src.collimator = float(rng.uniform(0.0, 90.0))
    blk = Block()
    if rect is None:
        blk.set_square(field)
    else:
        fx, fz = rng.uniform(rect[0], rect[1], size=2)
        blk.set_rect(-fx / 2, fx / 2, -fz / 2, fz / 2)
    return src, blk
