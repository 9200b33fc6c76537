"""Jaw/MLC transmission map in the isocentre plane.

Same contract as ``conehead/block.py:7-85``: ``block_values`` is a float32
transmission map sampled every 0.1 mm over [-20, 20) cm in both beam
directions (4000 x 4000).  Row index follows the beam x axis, column index
the beam z axis.  The dose kernels look a point (x, z) up as
``block_values[floor(100 x) + 1999, floor(100 z) + 1999]`` with the
reference's quirks (see ``transmission``).

``set_square`` reproduces the reference's integer truncation exactly.
``set_rect`` is an extension for asymmetric jaw fields (x1, x2, z1, z2 in cm
at the isocentre plane) built with the same truncation rule; the reference
only offers square fields and DICOM plans.
"""
import numpy as np


class Block:
    def __init__(self, rotation=np.array([0, 0, 0], dtype=np.float32), plan=None):
        self.rotation = rotation
        if plan is not None:
            raise NotImplementedError(
                "DICOM RT-plan blocking is not supported by this engine yet")
        self.xmin = np.float32(-20)
        self.xmax = np.float32(20)
        self.xnum = np.int32(4000)
        self.xres = self.xnum / (self.xmax - self.xmin)
        self.ymin = np.float32(-20)
        self.ymax = np.float32(20)
        self.ynum = np.int32(4000)
        self.yres = self.ynum / (self.ymax - self.ymin)
        self.block_values = np.zeros((self.xnum, self.ynum), dtype=np.float32)

    def transmission(self, position):
        """Transmission at an isocentre-plane point (cm), reference rules.

        The point is converted to 0.1 mm cells with ``floor(100 p) + 2000``;
        a cell index outside [0, 3999] gives 0, otherwise the map is read at
        ``index - 1`` (so index 0 wraps to the last row/column).
        """
        cell = np.floor(np.asarray(position, dtype=np.float32) * np.float32(100))
        cell = cell + np.float32(2000)
        for c in cell:
            if c < 0 or c > 3999:
                return np.float32(0)
        return self.block_values[int(cell[0]) - 1, int(cell[1]) - 1]

    def _open(self, x1, x2, y1, y2):
        self.block_values[x1:x2, y1:y2] = np.float32(1)

    def set_square(self, length):
        """Open a centred square of side ``length`` cm."""
        half = length / 2
        lo_x = int((self.xnum / 2) - half * self.xres)
        hi_x = int((self.xnum / 2) + half * self.xres)
        lo_y = int((self.ynum / 2) - half * self.yres)
        hi_y = int((self.ynum / 2) + half * self.yres)
        self._open(lo_x, hi_x, lo_y, hi_y)

    def set_rect(self, x1, x2, z1, z2):
        """Open the jaw rectangle [x1, x2] x [z1, z2] cm (x1 < x2, z1 < z2).

        Cell limits use the same ``int(n/2 + pos * res)`` truncation that
        ``set_square`` applies, so ``set_rect(-a/2, a/2, -a/2, a/2)`` equals
        ``set_square(a)``.
        """
        if not (x1 < x2 and z1 < z2):
            raise ValueError("set_rect needs x1 < x2 and z1 < z2")
        lo_x = int((self.xnum / 2) + x1 * self.xres)
        hi_x = int((self.xnum / 2) + x2 * self.xres)
        lo_y = int((self.ynum / 2) + z1 * self.yres)
        hi_y = int((self.ynum / 2) + z2 * self.yres)
        self._open(max(lo_x, 0), min(hi_x, int(self.xnum)),
                   max(lo_y, 0), min(hi_y, int(self.ynum)))
