"""EDKnrc polyenergetic energy-deposition kernel tables (host precompute).

Follows ``conehead/kernel.py:19-72`` and the table build in
``conehead/conehead.py:685-706``:

* ``KernelMono`` -- one monoenergetic run: 48 cone angles x 24 sphere radii
  of the ``total`` column, normalised to unit sum, cumulated over radius and
  resampled with linear interpolation onto r = 0.05 .. 60.0 cm in 0.1 mm
  steps (5996 points, float64).
* ``KernelPoly`` -- the spectrum-weighted mixture of mono ``kernel_diff``
  tables, normalised again and resampled the same way.
* ``poly_kernel_tables(energy_weights)`` -- what ``Conehead.calculate``
  uploads to the device: cumulative table K[48, 5996] (float64), the twelve
  azimuths theta = 0, 30, ..., 330 deg (float32) and the 48 cone polar
  angles phi (float32, 3.75 .. 180 deg).

Reference quirk kept on purpose: the "1.0" MeV spectrum bin is given the
1.5 MeV kernel (``conehead/conehead.py:688``).

Kernel data come from ``data/edknrc_6mv.npz`` (packed from conehead's
``kernels/*/*.egslst`` by ``data/extract_edknrc.py``) or, when
``kernel_dir`` is given, straight from the ``.egslst`` listings.
"""
import os
from functools import lru_cache

import numpy as np

N_CONES = 48
N_RADII = 24
N_SAMPLES = 5996          # 0.05 .. 60.0 cm every 0.1 mm
LABELS = ("0.5", "1.0", "1.5", "2.0", "2.5", "3.0",
          "3.5", "4.0", "4.5", "5.0", "5.5", "6.0")
# spectrum label -> kernel file label (reference loads 1.5 MeV for "1.0")
FILE_FOR_LABEL = {lab: lab for lab in LABELS}
FILE_FOR_LABEL["1.0"] = "1.5"

_PACKAGED = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                         "data", "edknrc_6mv.npz")


def _resample_cumulative(radii, kernel_cum):
    """Linear resample of each cone's cumulative curve onto the 0.1 mm grid."""
    r = np.linspace(0.05, 60.0, N_SAMPLES)
    out = np.zeros((kernel_cum.shape[0], N_SAMPLES))
    for cone in range(kernel_cum.shape[0]):
        out[cone, :] = np.interp(r, radii, kernel_cum[cone, :])
    return out


class KernelMono:
    """One monoenergetic EDKnrc kernel.

    ``KernelMono(path)`` parses an ``.egslst`` listing;
    ``KernelMono.from_raw(data_raw, energy)`` builds from an already parsed
    (1152, 3) float32 block (angle, radius, total).
    """

    def __init__(self, egslst_path=None):
        if egslst_path is None:
            raise NotImplementedError
        from .data.extract_edknrc import parse_egslst
        energy, data_raw = parse_egslst(egslst_path)
        self._build(data_raw, energy)

    @classmethod
    def from_raw(cls, data_raw, energy=None):
        obj = cls.__new__(cls)
        obj._build(np.asarray(data_raw, dtype=np.float32), energy)
        return obj

    def _build(self, data_raw, energy):
        self.energy = energy
        self.angles = np.unique(data_raw[:, 0])
        self.radii = np.unique(data_raw[:, 1])
        diff = data_raw[:, 2].reshape((N_CONES, N_RADII))
        self.kernel_diff = diff / diff.sum()
        self.kernel_cum = _resample_cumulative(
            self.radii, self.kernel_diff.cumsum(axis=1))


class KernelPoly:
    """Spectrum-weighted kernel built from already weighted ``kernel_diff``."""

    def __init__(self, angles, radii, kernel_diff):
        self.angles = angles
        self.radii = radii
        self.kernel_diff = kernel_diff / kernel_diff.sum()
        # the cumulative curve is taken from the argument, as the reference does
        self.kernel_cum = _resample_cumulative(radii, kernel_diff.cumsum(axis=1))


@lru_cache(maxsize=None)
def _packaged_monos():
    pack = np.load(_PACKAGED)
    return {lab: KernelMono.from_raw(pack[f"E{lab}"], float(pack[f"energy_{lab}"]))
            for lab in LABELS}


@lru_cache(maxsize=8)
def _dir_monos(kernel_dir):
    return {lab: KernelMono(os.path.join(kernel_dir, f"{lab}MeV", f"{lab}MeV.egslst"))
            for lab in LABELS}


def mono_kernels(kernel_dir=None):
    """Map spectrum label -> KernelMono, with the reference's file mapping."""
    files = _packaged_monos() if kernel_dir is None else _dir_monos(os.path.abspath(kernel_dir))
    return {lab: files[FILE_FOR_LABEL[lab]] for lab in LABELS}


def poly_kernel_tables(energy_weights, kernel_dir=None):
    """Return (K float64 [48, 5996], thetas float32 [12], phis float32 [48]).

    ``energy_weights`` is the settings dict {"0.5": w, ...}; keys must be
    spectrum labels.  Summation order follows the dict order, like the
    reference.
    """
    monos = mono_kernels(kernel_dir)
    first = monos["0.5"]
    diff = np.zeros_like(first.kernel_diff)
    for label, weight in energy_weights.items():
        if label not in monos:
            raise KeyError(f"no EDKnrc kernel for spectrum bin {label!r}")
        diff += monos[label].kernel_diff * weight
    diff = diff / diff.sum()
    poly = KernelPoly(first.angles, first.radii, diff)
    thetas = np.linspace(0, 360 - (360 / 12), 12, dtype=np.float32)
    return poly.kernel_cum, thetas, np.asarray(poly.angles, dtype=np.float32)
