"""Dose comparison against the CPU oracle, shared by the GPU parity tests.

Bars:
* against the float32-mirrored oracle: every voxel within ``DOSE_F32`` of
  Dmax (the GPU reproduces its float32 choices, so only summation order and
  float32 exp/FMA rounding differ);
* against the FP64 re-run: every voxel above 1% of Dmax within ``DOSE_BAR``
  (0.5% of Dmax), outside the neighbourhood of blocking flips.  A flip is a
  blocking sub-sample within float32 rounding of a 0.1 mm block-map cell
  edge: the FP64 re-run picks the neighbouring cell, so that voxel's blocked
  fraction moves by one sub-sample.  The reference computes in float32 and
  the GPU follows it bit for bit there; the flip voxels are counted and their
  error reported, not hidden.
"""
import numpy as np

DOSE_BAR = 5e-3
DOSE_F32 = 2e-4


def near_flips(ref32, ref64):
    flip = ref32["blocked"] != ref64["blocked"]
    near = flip.copy()
    for ax in range(3):
        for sh in (-1, 1):
            near |= np.roll(flip, sh, axis=ax)
    return flip, near


def check_dose(oracle_lib, dose, source, block, phantom, settings, label, f64=True):
    """Compare a GPU dose (numpy float32 [x][y][z]), or a dict of named GPU
    doses of the same beam, with the oracle run once on the same inputs;
    asserts the bars and returns one summary line per dose with the
    measured errors."""
    doses = dose if isinstance(dose, dict) else {label: dose}
    ref = oracle_lib.calculate(source, block, phantom, settings, oracle_lib.MODE_F32)
    D32 = ref["dose"]
    assert D32.max() > 0, f"{label}: zero reference dose"
    ref64 = oracle_lib.calculate(source, block, phantom, settings, oracle_lib.MODE_F64) if f64 else None
    lines = []
    for name, d in doses.items():
        e32 = np.abs(d.astype(np.float64) - D32).max() / D32.max()
        msg = f"{name}: vs fp32-mirrored oracle {e32:.2e} of Dmax"
        assert e32 <= DOSE_F32, msg
        if f64:
            flip, near = near_flips(ref, ref64)
            D = ref64["dose"]
            hot = (D > 0.01 * D.max()) & ~near
            err = np.abs(d.astype(np.float64) - D)
            e64 = err[hot].max() / D.max()
            msg += f", vs FP64 oracle {e64:.2e} of Dmax (all voxels {err.max() / D.max():.2e})"
            if flip.any():
                msg += (f"; {int(flip.sum())} voxel(s) with a float32/float64 blocking flip, "
                        f"{err[near].max() / D.max():.2e} of Dmax there")
            assert e64 <= DOSE_BAR, msg
        print(msg)
        lines.append(msg)
    return lines
