"""Device-resident dose engine over the C ABI.

``DoseEngine`` owns one ``ch_plan`` (kernel tables, direction stencils and
scratch stay on the GPU between calls) and runs single beams, batches of
beams and the plain scatter path on torch CUDA tensors.  Host objects use
the reference's duck-typed attributes (``source.position/v_y/transform/
sad``, ``block.block_values``, ``phantom.size/origin/spacing/densities``)
and its ``settings`` dict.
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .kernel import poly_kernel_tables


@dataclass
class DeviceBlock:
    """Block map on the device, cropped to its nonzero bounding box."""
    crop: object          # torch float32 tensor [rows, cols]; None for a uniform crop
    r0: int
    c0: int
    full_shape: tuple
    uniform: bool = False  # every crop value is 1.0 (a jaw rectangle)
    shape: tuple = None    # crop shape when there is no tensor
    zero: bool = False     # nothing open: a 1 x 1 crop of zeros

    def __post_init__(self):
        if self.crop is not None:
            self.shape = tuple(self.crop.shape)
        elif self.zero:
            self.uniform = False


@dataclass
class BeamJob:
    grid: object          # N.Grid
    rho: object           # torch float32 tensor, phantom.densities layout
    swap_xy: int
    beam: object          # N.Beam
    settings: object      # N.Settings
    dose: object          # torch float32 tensor [nx, ny, nz]
    keep: tuple = ()      # tensors the beam struct points at


class DoseEngine:
    def __init__(self, device=0):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("conehead_gb300 needs a CUDA GPU (GB300); no CPU fallback exists")
        self.torch = torch
        self.index = int(device)
        self.device = torch.device("cuda", self.index)
        self.L = N.lib()
        plan = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            N.check(self.L.ch_plan_create(ctypes.byref(plan), self.index), "ch_plan_create")
        self.plan = plan
        self._kernel_key = None

    def close(self):
        if getattr(self, "plan", None):
            self.L.ch_plan_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ set-up --
    def stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream(self.device).cuda_stream)

    def set_kernel(self, energy_weights, kernel_dir=None):
        key = (tuple((k, float(v)) for k, v in energy_weights.items()), kernel_dir)
        if key == self._kernel_key:
            return
        K, thetas, phis = poly_kernel_tables(energy_weights, kernel_dir)
        K = np.ascontiguousarray(K, dtype=np.float64)
        thetas = np.ascontiguousarray(thetas, dtype=np.float32)
        phis = np.ascontiguousarray(phis, dtype=np.float32)
        k = N.Kernel(K.shape[0], K.shape[1], len(thetas), K.ctypes.data, thetas.ctypes.data,
                     phis.ctypes.data)
        N.check(self.L.ch_plan_set_kernel(self.plan, ctypes.byref(k)), "ch_plan_set_kernel")
        self._kernel_key = key

    def upload_block(self, block_values):
        crop, r0, c0 = N.block_crop(block_values)
        t = self.torch.from_numpy(crop).to(self.device)
        return DeviceBlock(t, r0, c0, tuple(np.shape(block_values)), bool(np.all(crop == 1.0)))

    def upload_mlc(self, mlc):
        """Rasterise the jaw opening of an MLC map on the device (no host map)."""
        r0, r1, c0, c1 = mlc.window
        full = (mlc.rows, 4000)
        if r1 <= r0 or c1 <= c0:
            return DeviceBlock(self.torch.zeros((1, 1), dtype=self.torch.float32, device=self.device), 0, 0, full)
        crop = self.torch.empty((r1 - r0, c1 - c0), dtype=self.torch.float32, device=self.device)
        m = mlc.struct()
        N.check(self.L.ch_block_from_mlc(ctypes.byref(m), crop.data_ptr(), r1 - r0, c1 - c0, r0, c0,
                                         self.stream()), "ch_block_from_mlc")
        return DeviceBlock(crop, r0, c0, full)

    def jaw_block(self, rect, full_shape=(4000, 4000)):
        """A rectangle of ones: no memory at all, the kernels read the flag."""
        r0, r1, c0, c1 = rect
        if r1 <= r0 or c1 <= c0:
            return DeviceBlock(None, 0, 0, full_shape, True, (1, 1), zero=True)
        return DeviceBlock(None, r0, c0, full_shape, True, (r1 - r0, c1 - c0))

    def block_for(self, block):
        """Device block of a Block-like object.  Blocks whose map was never read
        on the host go to the GPU as what they are -- a jaw rectangle (a
        uniform crop, no memory) or a leaf table (rasterised on the device);
        anything else is cropped from ``block_values``."""
        rect = getattr(block, "device_rect", None)
        rect = rect() if callable(rect) else None
        if rect is not None:
            return self.jaw_block(rect, (int(block.xnum), int(block.ynum)))
        table = getattr(block, "device_mlc", None)
        mlc = table() if callable(table) else None
        if mlc is not None:
            return self.upload_mlc(mlc)
        return self.upload_block(block.block_values)

    def upload_densities(self, densities):
        return self.torch.from_numpy(np.ascontiguousarray(densities, dtype=np.float32)).to(self.device)

    def job(self, phantom, rho, source, dblock, settings, swap_xy=None, dose=None):
        size = [int(n) for n in phantom.size]
        if swap_xy is None:
            swap_xy = int(size[0] == size[1])
        grid = N.grid_struct(size, phantom.origin, phantom.spacing)
        if dblock.zero:
            if getattr(self, "_zero_crop", None) is None:
                self._zero_crop = self.torch.zeros((1, 1), dtype=self.torch.float32, device=self.device)
            dblock = DeviceBlock(self._zero_crop, 0, 0, dblock.full_shape)
        ptr = dblock.crop.data_ptr() if dblock.crop is not None else None
        beam = N.beam_struct(source, ptr, dblock.shape, dblock.r0, dblock.c0,
                             dblock.full_shape, dblock.uniform)
        s = settings if isinstance(settings, N.Settings) else self._settings(settings)
        if dose is None:
            dose = self.torch.empty(size, dtype=self.torch.float32, device=self.device)
        return BeamJob(grid, rho, int(swap_xy), beam, s, dose, (dblock.crop,))

    def _settings(self, settings):
        """ch_settings of a settings dict, cached on its contents."""
        try:
            key = tuple((k, tuple(v.items()) if isinstance(v, dict) else v) for k, v in sorted(settings.items()))
            hash(key)
        except TypeError:
            return N.settings_struct(settings)
        cache = self.__dict__.setdefault("_settings_cache", {})
        s = cache.get(key)
        if s is None:
            if len(cache) > 64:
                cache.clear()
            s = cache[key] = N.settings_struct(settings)
        return s

    # ----------------------------------------------------------- compute --
    def run(self, job, intermediates=False, scatter=False):
        """Enqueue one beam; returns the dose tensor (and intermediates)."""
        torch = self.torch
        st = self.stream()
        out = None
        if scatter:
            N.check(self.L.ch_dose_scatter(self.plan, ctypes.byref(job.grid), job.rho.data_ptr(), job.swap_xy,
                                           ctypes.byref(job.beam), ctypes.byref(job.settings),
                                           job.dose.data_ptr(), st), "ch_dose_scatter")
        elif intermediates:
            size = list(job.dose.shape)
            out = {"blocked": torch.empty(size, dtype=torch.float64, device=self.device)}
            for k in ("d_eff", "oad", "fluence", "f_soften", "f_horn", "terma"):
                out[k] = torch.empty(size, dtype=torch.float32, device=self.device)
            inter = N.Intermediates(*[out[k].data_ptr() for k in
                                      ("blocked", "d_eff", "oad", "fluence", "f_soften", "f_horn", "terma")])
            N.check(self.L.ch_dose_ex(self.plan, ctypes.byref(job.grid), job.rho.data_ptr(), job.swap_xy,
                                      ctypes.byref(job.beam), ctypes.byref(job.settings), job.dose.data_ptr(),
                                      ctypes.byref(inter), st), "ch_dose_ex")
        else:
            N.check(self.L.ch_dose(self.plan, ctypes.byref(job.grid), job.rho.data_ptr(), job.swap_xy,
                                   ctypes.byref(job.beam), ctypes.byref(job.settings), job.dose.data_ptr(), st),
                    "ch_dose")
        return (job.dose, out) if intermediates else job.dose

    def run_batch(self, jobs):
        """Enqueue many beams in one pass; returns their dose tensors."""
        n = len(jobs)
        grids = (N.Grid * n)(*[j.grid for j in jobs])
        beams = (N.Beam * n)(*[j.beam for j in jobs])
        sets = (N.Settings * n)(*[j.settings for j in jobs])
        rho = (ctypes.c_void_p * n)(*[j.rho.data_ptr() for j in jobs])
        dose = (ctypes.c_void_p * n)(*[j.dose.data_ptr() for j in jobs])
        swap = (ctypes.c_int * n)(*[j.swap_xy for j in jobs])
        N.check(self.L.ch_dose_batch(self.plan, n, grids, rho, swap, beams, sets, dose, self.stream()),
                "ch_dose_batch")
        return [j.dose for j in jobs]

    def sync(self):
        N.check(self.L.ch_plan_sync(self.plan, self.stream()), "ch_plan_sync")

    # ---------------------------------------------------------- schedule --
    def set_tuning(self, dir_group=16, unit_order=0, terma_ctas_per_sm=8, cone_method=N.CONE_SPECTRAL):
        """Schedule knobs (``ch_tuning``); cone_method 0 = spectral, 1 = gather."""
        t = N.Tuning(int(dir_group), int(unit_order), int(terma_ctas_per_sm), int(cone_method))
        N.check(self.L.ch_plan_set_tuning(self.plan, ctypes.byref(t)), "ch_plan_set_tuning")

    def get_tuning(self):
        t = N.Tuning()
        N.check(self.L.ch_plan_get_tuning(self.plan, ctypes.byref(t)), "ch_plan_get_tuning")
        return {k: getattr(t, k) for k, _ in N.Tuning._fields_}

    def set_wait_limit(self, iterations=0, withhold=0):
        """Bound of the gather's pipeline waits (try_wait iterations; 0 = the
        default) and the test hook of their expiry (``withhold`` 1: no window
        is issued; 2: no slot is freed; 0: off)."""
        N.check(self.L.ch_plan_set_wait_limit(self.plan, int(iterations), int(withhold)),
                "ch_plan_set_wait_limit")

    def prepare(self, size, spacing):
        """Build the stencils for grids up to ``size`` at ``spacing`` now."""
        g = N.grid_struct(size, (0.0, 0.0, 0.0), spacing)
        N.check(self.L.ch_plan_prepare(self.plan, ctypes.byref(g), self.stream()), "ch_plan_prepare")

    def capture(self, jobs):
        """A CapturedBatch of these jobs (one CUDA graph, replayed by launch())."""
        return CapturedBatch(self, jobs)

    def stats(self):
        s = N.Stats()
        N.check(self.L.ch_plan_stats(self.plan, ctypes.byref(s)), "ch_plan_stats")
        return {k: getattr(s, k) for k, _ in N.Stats._fields_}

    # ------------------------------------------------------- test hooks --
    def cone_directions(self):
        import torch
        n = 12 * 48
        out = torch.empty((n, 3), dtype=torch.float32, device=self.device)
        N.check(self.L.ch_cone_directions(self.plan, out.data_ptr(), self.stream()), "ch_cone_directions")
        self.sync()
        return out.cpu().numpy()


class CapturedBatch:
    """ch_batch: the jobs' device work captured once into a CUDA graph.

    ``launch()`` recomputes every job's dose from the current contents of its
    density and block-map tensors; geometry, settings and grids are fixed.
    The jobs' tensors must stay alive and in place while the batch exists.
    """

    def __init__(self, engine, jobs):
        self.eng = engine
        self.jobs = list(jobs)
        n = len(self.jobs)
        grids = (N.Grid * n)(*[j.grid for j in self.jobs])
        beams = (N.Beam * n)(*[j.beam for j in self.jobs])
        sets = (N.Settings * n)(*[j.settings for j in self.jobs])
        rho = (ctypes.c_void_p * n)(*[j.rho.data_ptr() for j in self.jobs])
        dose = (ctypes.c_void_p * n)(*[j.dose.data_ptr() for j in self.jobs])
        swap = (ctypes.c_int * n)(*[j.swap_xy for j in self.jobs])
        h = ctypes.c_void_p()
        N.check(engine.L.ch_batch_create(engine.plan, n, grids, rho, swap, beams, sets, dose, engine.stream(),
                                         ctypes.byref(h)), "ch_batch_create")
        self.handle = h

    def launch(self):
        N.check(self.eng.L.ch_batch_launch(self.handle, self.eng.stream()), "ch_batch_launch")
        return [j.dose for j in self.jobs]

    def sync(self):
        N.check(self.eng.L.ch_batch_sync(self.handle, self.eng.stream()), "ch_batch_sync")

    def close(self):
        if getattr(self, "handle", None):
            self.eng.L.ch_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dda_trace(size, spacing, starts, dirs, cap=1024, device=0):
    """Device DDA traces (test hook): voxels [n, cap, 3], t [n, cap], lengths [n]."""
    import torch
    dev = torch.device("cuda", device)
    starts = torch.as_tensor(np.ascontiguousarray(starts, dtype=np.int32), device=dev)
    dirs = torch.as_tensor(np.ascontiguousarray(dirs, dtype=np.float32), device=dev)
    n = starts.shape[0]
    vox = torch.zeros((n, cap, 3), dtype=torch.int32, device=dev)
    tv = torch.zeros((n, cap), dtype=torch.float32, device=dev)
    ln = torch.zeros((n,), dtype=torch.int32, device=dev)
    g = N.grid_struct(size, (0, 0, 0), spacing)
    st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    N.check(N.lib().ch_dda_trace(ctypes.byref(g), n, starts.data_ptr(), dirs.data_ptr(), cap, vox.data_ptr(),
                                 tv.data_ptr(), ln.data_ptr(), st), "ch_dda_trace")
    torch.cuda.synchronize(dev)
    return vox.cpu().numpy(), tv.cpu().numpy(), ln.cpu().numpy()
