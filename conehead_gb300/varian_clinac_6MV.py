"""6 MV Varian Clinac photon spectrum models (``conehead/varian_clinac_6MV.py``).

The dose path itself takes its spectrum from ``settings['energy_weights']``;
these analytic/tabulated spectra are helpers for building that dict
(``spectrum_weights``).

* ``weights_ali`` -- Ali & Rogers 2012 (Phys. Med. Biol. 57 31), eq. 12 with
  the table-5 Clinac 6 MV constants: a thin-target bremsstrahlung shape
  hardened by 1.222 cm of tungsten and 5.147 cm of aluminium, normalised by
  the trapezoid rule when given an array.
* ``weights_cho`` -- lognormal generic 6 MV spectrum (Cho et al 2012).
* ``weights_sheikh_bagheri`` -- tabulated Sheikh-Bagheri & Rogers 2002
  spectrum, cubic interpolation, normalised to unit area.
"""
import numpy as np
from scipy.interpolate import interp1d

from .nist import mu_Al, mu_W


def _trapezoid(y, x):
    y = np.asarray(y, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    return float(np.sum((x[1:] - x[:-1]) * (y[1:] + y[:-1]) / 2.0))


def weights_cho(E):
    mu, sigma = 0.30, 0.8
    w = 1 / (np.sqrt(2 * np.pi) * sigma * E)
    w *= np.exp(-np.power(np.log(E) - mu, 2) / (2 * np.power(sigma, 2)))
    return w


def weights_ali(E):
    c1, c2, c3, e_e = 1.222, 5.147, -1.186, 5.76
    ratio = E / e_e
    # above the endpoint energy the logarithm's argument is negative: NaN,
    # and those weights are zero below
    with np.errstate(invalid="ignore"):
        thin = (1 + c3 * ratio + np.power(ratio, 2)) * \
            (np.log(e_e * (e_e - E) / E + 1.65) - 0.5)
    psi = thin * np.exp(-mu_W(E) * np.power(c1, 2) - mu_Al(E) * np.power(c2, 2))
    if isinstance(psi, np.ndarray) and psi.ndim > 0:
        psi[psi < 0] = 0
        psi /= _trapezoid(psi, E)
        return psi
    psi = float(psi)
    if psi < 0 or np.isnan(psi):
        psi = 0
    return np.array(psi, dtype=np.float32)


_SB_TABLE = (
    (0.250, 0.214e-4), (0.500, 0.126e-3), (0.750, 0.131e-3), (1.000, 0.114e-3),
    (1.250, 0.976e-4), (1.500, 0.836e-4), (1.750, 0.725e-4), (2.000, 0.623e-4),
    (2.250, 0.535e-4), (2.500, 0.459e-4), (2.750, 0.395e-4), (3.000, 0.347e-4),
    (3.250, 0.298e-4), (3.500, 0.261e-4), (3.750, 0.225e-4), (4.000, 0.191e-4),
    (4.250, 0.166e-4), (4.500, 0.138e-4), (4.750, 0.114e-4), (5.000, 0.904e-5),
    (5.250, 0.655e-5), (5.500, 0.409e-5), (5.750, 0.140e-5), (6.000, 0.434e-7),
)


def weights_sheikh_bagheri(E):
    table = np.array(_SB_TABLE)
    table[:, 1] /= _trapezoid(table[:, 1], table[:, 0])
    return interp1d(table[:, 0], table[:, 1], bounds_error=False,
                    kind="cubic", fill_value=0)(E)


def spectrum_weights(model=weights_ali, labels=("0.5", "1.0", "1.5", "2.0", "2.5",
                                                "3.0", "3.5", "4.0", "4.5", "5.0",
                                                "5.5", "6.0")):
    """Build an ``energy_weights`` settings dict from a spectrum model."""
    energies = np.array([float(lab) for lab in labels], dtype=np.float32)
    w = np.asarray(model(energies), dtype=np.float64)
    w = np.where(np.isfinite(w), w, 0.0)
    return {lab: float(v) for lab, v in zip(labels, w)}
