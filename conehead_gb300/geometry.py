"""Line / blocking-plane intersection (``conehead/geometry.py:105-134``).

The blocking plane passes through the isocentre (the world origin) with
normal ``plane_normal`` (the beam axis ``source.v_y``).  A ray nearly
parallel to it (|n . u| < epsilon) has no usable intersection and raises
RuntimeError, as the reference does.
"""
import numpy as np


def line_block_plane_collision(ray_start, ray_direction, plane_normal, epsilon=1e-6):
    plane_point = np.array([0, 0, 0], dtype=np.float32)
    ndotu = plane_normal.dot(ray_direction)
    if abs(ndotu) < epsilon:
        raise RuntimeError("no intersection or line is within plane")
    w = ray_start - plane_point
    si = -plane_normal.dot(w) / ndotu
    return w + si * ray_direction + plane_point
