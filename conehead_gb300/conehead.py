"""``Conehead.calculate`` -- drop-in for conehead/conehead.py:520-738.

Same class name, same call ``Conehead().calculate(source, block, phantom,
settings)`` with the reference's duck-typed objects and settings dict.
Differences, all deliberate:

* the dose is returned (float32 numpy [nx, ny, nz]) and stored in
  ``self.dose_grid.dose``; the reference leaves it in a local variable and
  returns None;
* no progress prints and no matplotlib figure;
* the EDKnrc kernels come from the packaged tables (or ``kernel_dir``), not
  from paths relative to the working directory;
* ``return_intermediates=True`` also returns blocked, d_eff, oad, fluence,
  f_soften, f_horn and TERMA.

Everything runs on the GPU through the CUDA library; nothing falls back to
the CPU.  The density resampling step of the reference (scipy
RegularGridInterpolator evaluated at its own nodes with meshgrid's default
'xy' indexing) is exactly a transpose of x and y, which the kernels apply by
reading the densities with x and y swapped when nx == ny (for nx != ny the
reference reads out of bounds; here the densities are then read as given).
"""
import numpy as np

from .phantom import DoseGrid

_ENGINES = {}


def engine(device=0):
    """Process-wide engine per CUDA device (plans keep tables resident)."""
    from .engine import DoseEngine
    if device not in _ENGINES:
        _ENGINES[device] = DoseEngine(device)
    return _ENGINES[device]


class Conehead:
    def __init__(self, device=0, kernel_dir=None):
        self.device = device
        self.kernel_dir = kernel_dir
        self.dose_grid = None

    def calculate(self, source, block, phantom, settings, return_intermediates=False):
        eng = engine(self.device)
        eng.set_kernel(settings["energy_weights"], self.kernel_dir)
        self.dose_grid = DoseGrid(phantom.size, phantom.origin, phantom.spacing)
        rho = eng.upload_densities(phantom.densities)
        dblock = eng.block_for(block)
        job = eng.job(phantom, rho, source, dblock, settings)
        if return_intermediates:
            dose, inter = eng.run(job, intermediates=True)
        else:
            dose, inter = eng.run(job), None
        eng.sync()
        self.dose_grid.dose = dose.cpu().numpy()
        if not return_intermediates:
            return self.dose_grid.dose
        out = {k: v.cpu().numpy() for k, v in inter.items()}
        out["dose"] = self.dose_grid.dose
        return out

    def calculate_batch(self, beams, phantom, settings):
        """Several beams on one phantom in one GPU pass.

        ``beams`` is a list of (source, block) pairs; returns a list of dose
        arrays in the same order.
        """
        eng = engine(self.device)
        eng.set_kernel(settings["energy_weights"], self.kernel_dir)
        rho = eng.upload_densities(phantom.densities)
        jobs = [eng.job(phantom, rho, src, eng.block_for(blk), settings)
                for src, blk in beams]
        doses = eng.run_batch(jobs)
        eng.sync()
        return [d.cpu().numpy() for d in doses]
