"""Phantom and dose-grid containers (``conehead/phantom.py``, ``conehead/dosegrid.py``).

The dose path reads ``size`` (three ints), ``origin`` and ``spacing``
(float32[3], cm; voxel *centres* sit at ``origin + spacing * index``) and
``densities`` (float32, shape ``size``, g/cc, C order ``[x, y, z]``).
"""
import numpy as np


class SimplePhantom:
    """40 cm water cube, 201^3 voxels of 2 mm, surface on the isocentre plane."""

    def __init__(self):
        self.size = [201, 201, 201]
        self.origin = np.array([-20.1, 0, -20.1], dtype=np.float32)
        self.spacing = np.array([.2, .2, .2], dtype=np.float32)
        self.densities = np.ones(self.size, dtype=np.float32)


class GridPhantom:
    """Arbitrary phantom: any size, origin, spacing and density array."""

    def __init__(self, densities, origin, spacing):
        self.densities = np.ascontiguousarray(densities, dtype=np.float32)
        self.size = [int(n) for n in self.densities.shape]
        self.origin = np.asarray(origin, dtype=np.float32)
        self.spacing = np.asarray(spacing, dtype=np.float32)


class DoseGrid:
    def __init__(self, size, origin, spacing):
        self.size = size
        self.origin = origin
        self.spacing = spacing
        self.dose = np.zeros(self.size, dtype=np.float32)
