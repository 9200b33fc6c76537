"""Beamlet-weight gradients of the dose: the hand-written adjoint.

A beamlet fluence map is a rows x cols grid of beamlets on the block map
(0.1 mm cells), each holding one weight; its dose is exactly the reference's
dose for that block map (conehead/conehead.py:522-738), computed by the
forward engine.  The gradient of any scalar objective of the dose with
respect to the weights runs on the GPU through ``ch_dose_adjoint``:

* dL/dTERMA = C^T dL/dD: the transposed collapsed-cone stage, the same
  stencil gather along the mirrored walks (no atomics but one add per output
  and work unit), computed only where TERMA is nonzero;
* dL/dw: TERMA = blocked^2 * H(v) (fluence and TERMA each carry one factor of
  the blocked fraction, conehead/conehead.py:641-662), and blocked(v) is the
  mean of w over the beamlets hit by the voxel's S^3 sub-samples
  (conehead/conehead.py:71-120), so every sub-sample adds
  2 T(v)/blocked(v) * dL/dT(v) / S^3 to its beamlet -- the transposed ray
  trace from voxel to block plane, with the exact float64 projection
  wherever a sub-sample sits within float32 error of a beamlet edge.

``BeamletDose`` wraps both directions for one beam and phantom;
``beamlet_dose(weights, op)`` is the ``torch.autograd.Function`` entry.
"""
import ctypes

import numpy as np

from . import _native as N

MAP = 4000          # block map cells per side (0.1 mm)


class BeamletGrid:
    """rows x cols beamlets of cell x cell map cells, centred on the map."""

    def __init__(self, rows, cols, cell_rows, cell_cols=None, r0=None, c0=None):
        self.rows, self.cols = int(rows), int(cols)
        self.cell_rows = int(cell_rows)
        self.cell_cols = int(cell_cols if cell_cols is not None else cell_rows)
        self.r0 = int(r0) if r0 is not None else MAP // 2 - self.rows * self.cell_rows // 2
        self.c0 = int(c0) if c0 is not None else MAP // 2 - self.cols * self.cell_cols // 2
        if not (0 <= self.r0 and self.r0 + self.rows * self.cell_rows <= MAP and
                0 <= self.c0 and self.c0 + self.cols * self.cell_cols <= MAP):
            raise ValueError("beamlet grid does not fit the 4000 x 4000 block map")

    @classmethod
    def square(cls, n, beamlet_cm):
        """n x n beamlets of beamlet_cm (0.5 cm = 50 map cells)."""
        cell = int(round(beamlet_cm * 100))
        return cls(n, n, cell)

    @property
    def shape(self):
        return (self.rows, self.cols)

    @property
    def crop_shape(self):
        return (self.rows * self.cell_rows, self.cols * self.cell_cols)

    def struct(self):
        return N.Beamlets(self.rows, self.cols, self.cell_rows, self.cell_cols, self.r0, self.c0)

    def host_map(self, weights):
        """The full float32 block map of these weights (for the oracle)."""
        w = np.asarray(weights, dtype=np.float32).reshape(self.rows, self.cols)
        m = np.zeros((MAP, MAP), dtype=np.float32)
        crop = np.repeat(np.repeat(w, self.cell_rows, axis=0), self.cell_cols, axis=1)
        m[self.r0:self.r0 + crop.shape[0], self.c0:self.c0 + crop.shape[1]] = crop
        return m


class MapBlock:
    """A Block-like holder of a host block map (what the oracle reads)."""

    def __init__(self, values):
        self.block_values = values


class BeamletDose:
    """Dose of one beam on one phantom as a function of beamlet weights."""

    def __init__(self, engine, phantom, source, beamlets, settings):
        import torch
        self.torch = torch
        self.eng = engine
        self.phantom = phantom
        self.source = source
        self.beamlets = beamlets
        self.settings = settings
        engine.set_kernel(settings["energy_weights"])
        self.rho = engine.upload_densities(phantom.densities)
        self.bl = beamlets.struct()
        self.crop = torch.empty(beamlets.crop_shape, dtype=torch.float32, device=engine.device)
        self.size = tuple(int(n) for n in phantom.size)

    def _job(self, dose=None):
        from .engine import DeviceBlock
        db = DeviceBlock(self.crop, self.beamlets.r0, self.beamlets.c0, (MAP, MAP), False)
        return self.eng.job(self.phantom, self.rho, self.source, db, self.settings, dose=dose)

    def _fill(self, weights):
        w = weights.detach().to(device=self.eng.device, dtype=self.torch.float32).contiguous()
        if tuple(w.shape) != self.beamlets.shape:
            raise ValueError(f"weights must have shape {self.beamlets.shape}")
        N.check(self.eng.L.ch_block_from_beamlets(ctypes.byref(self.bl), w.data_ptr(), self.crop.data_ptr(),
                                                  self.eng.stream()), "ch_block_from_beamlets")
        return w

    def forward(self, weights):
        """Dose (device float32 [nx, ny, nz]) of these weights."""
        self._fill(weights)
        job = self._job()
        self.eng.run(job)
        return job.dose

    def backward(self, grad_dose, weights=None, grad_terma=None):
        """dL/dw (device float32 [rows, cols]) for dL/d(dose) = grad_dose, at
        the weights of the last forward (or ``weights``)."""
        torch = self.torch
        if weights is not None:
            self._fill(weights)
        g = grad_dose.detach().to(device=self.eng.device, dtype=torch.float32).contiguous()
        if tuple(g.shape) != self.size:
            raise ValueError(f"grad_dose must have shape {self.size}")
        out = torch.empty(self.beamlets.shape, dtype=torch.float32, device=self.eng.device)
        job = self._job(dose=g)          # the dose slot is unused by the adjoint
        gt = grad_terma.data_ptr() if grad_terma is not None else None
        N.check(self.eng.L.ch_dose_adjoint(self.eng.plan, ctypes.byref(job.grid), self.rho.data_ptr(), job.swap_xy,
                                           ctypes.byref(job.beam), ctypes.byref(self.bl), ctypes.byref(job.settings),
                                           g.data_ptr(), out.data_ptr(), gt, self.eng.stream()), "ch_dose_adjoint")
        return out


def _function():
    import torch

    class BeamletDoseFunction(torch.autograd.Function):
        """dose = op.forward(weights); backward through ch_dose_adjoint."""

        @staticmethod
        def forward(ctx, weights, op):
            ctx.op = op
            ctx.save_for_backward(weights)
            return op.forward(weights)

        @staticmethod
        def backward(ctx, grad_dose):
            (weights,) = ctx.saved_tensors
            grad = ctx.op.backward(grad_dose, weights=weights)
            return grad.to(weights.dtype).to(weights.device), None

    return BeamletDoseFunction


_FN = None


def beamlet_dose(weights, op):
    """Differentiable dose of a BeamletDose operator at ``weights``."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(weights, op)


def cone(engine, grid_size, spacing, volume, transpose=False):
    """C volume or C^T volume (device float32 [x][y][z]) for this spacing."""
    import torch
    v = volume.contiguous()
    out = torch.empty_like(v)
    g = N.grid_struct(grid_size, (0.0, 0.0, 0.0), spacing)
    N.check(engine.L.ch_cone(engine.plan, ctypes.byref(g), v.data_ptr(), out.data_ptr(), int(bool(transpose)),
                             engine.stream()), "ch_cone")
    return out


def sphere_target(phantom, centre_cm, radius_cm, value=2.0):
    """Target dose: ``value`` inside a sphere (voxel centres), 0 elsewhere."""
    n = [int(k) for k in phantom.size]
    axes = [np.float32(phantom.origin[k]) + np.float32(phantom.spacing[k]) * np.arange(n[k], dtype=np.float32)
            for k in range(3)]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    r2 = (X - centre_cm[0]) ** 2 + (Y - centre_cm[1]) ** 2 + (Z - centre_cm[2]) ** 2
    return np.where(r2 <= radius_cm ** 2, np.float32(value), np.float32(0)).astype(np.float32)
