"""Point-source beam geometry (IEC 61217 gantry/collimator).

Mirrors the attribute contract of ``conehead/source.py:5-111`` because the
dose path reads these attributes directly:

* ``position``  -- source position in world coordinates (cm).  float32
  ``[0, -SAD, 0]`` until an angle is set, float64 afterwards (the reference
  rebuilds it from float64 trigonometry, conehead/source.py:80-85).
* ``v_x, v_y, v_z`` -- beam basis; ``v_y`` points from the source through
  the isocentre and is the normal of the blocking (isocentre) plane.
* ``transform`` -- world -> beam rotation, the matrix inverse of the basis
  ``[v_x v_y v_z]`` (conehead/source.py:110-111).  It is computed with
  ``numpy.linalg.inv`` rather than a transpose because the dose kernels use
  its exact float64 bits when projecting sample points into the block map.

The float32/float64 dtype switch matters: the reference's GPU kernels do the
plane projection in float32 for a fresh source and in float64 once an angle
has been set, and the engine reproduces both.
"""
import numpy as np


class Source:
    def __init__(self, model="varian_clinac_6MV", sad=np.float32(100)):
        if model != "varian_clinac_6MV":
            raise NotImplementedError(
                "The requested model is not yet implemented.")
        from . import varian_clinac_6MV
        self.weights = varian_clinac_6MV.weights_ali
        self._sad = sad
        self._gantry = 0
        self._collimator = 0
        self._position = np.array([0, -self._sad, 0], dtype=np.float32)
        self.v_x = np.array([1, 0, 0], dtype=np.float32)
        self.v_y = np.array([0, 1, 0], dtype=np.float32)
        self.v_z = np.array([0, 0, 1], dtype=np.float32)
        self.transform = np.linalg.inv(
            np.array([self.v_x, self.v_y, self.v_z]).transpose())

    # -- attributes -------------------------------------------------------
    @property
    def position(self):
        return self._position

    @position.setter
    def position(self, value):
        self._position = value

    @property
    def sad(self):
        return self._sad

    @property
    def gantry(self):
        return self._gantry

    @gantry.setter
    def gantry(self, angle):
        assert 0 <= angle < 360, "Invalid gantry angle"
        self._gantry = angle
        self._rebuild()

    @property
    def collimator(self):
        return self._collimator

    @collimator.setter
    def collimator(self, angle):
        assert 0 <= angle < 360, "Invalid collimator angle"
        self._collimator = angle
        self._rebuild()

    # -- geometry ---------------------------------------------------------
    def _rebuild(self):
        # IEC 61217: gantry g puts the source at polar angle (90 - g) in the
        # x-y plane, measured so that g = 0 is at (0, -SAD, 0).
        polar = (90 - self._gantry) % 360
        rad = polar * np.pi / 180
        self.position = np.array([self.sad * np.cos(rad),
                                  self.sad * -np.sin(rad),
                                  self.position[2]])
        ex = np.array([1, 0, 0], dtype=np.float32)
        ey = np.array([0, 1, 0], dtype=np.float32)
        ez = np.array([0, 0, 1], dtype=np.float32)
        # collimator: rotation about the beam (y) axis by -collimator
        c = -self._collimator * np.pi / 180
        rot_coll = np.array([[np.cos(c), 0, np.sin(c)],
                             [0, 1, 0],
                             [-np.sin(c), 0, np.cos(c)]])
        # gantry: rotation about the world z axis by +gantry
        g = self._gantry * np.pi / 180
        rot_gan = np.array([[np.cos(g), -np.sin(g), 0],
                            [np.sin(g), np.cos(g), 0],
                            [0, 0, 1]])
        self.v_x = np.matmul(rot_gan, np.matmul(rot_coll, ex))
        self.v_y = np.matmul(rot_gan, ey)
        self.v_z = np.matmul(rot_gan, np.matmul(rot_coll, ez))
        self.transform = np.linalg.inv(
            np.array([self.v_x, self.v_y, self.v_z]).transpose())
