"""ctypes binding of the engine's C ABI (include/conehead_gb300.h).

The CUDA library is the only compute path: if it is missing or cannot be
loaded, everything here raises -- there is no CPU fallback.  Device memory
and streams come from PyTorch (plumbing only); raw pointers are handed to
the library.
"""
import ctypes
import os

import numpy as np

from .build import LIB

CH_MAX_ENERGY = 32
CH_MAX_LEAF_PAIRS = 256
CH_MLC_TIP_CELLS = 15

STATUS = {0: "ok", 1: "invalid argument", 2: "out of device memory", 3: "CUDA error",
          4: "device wait timed out", 5: "ray parallel to the blocking plane",
          6: "kernel tables not set"}


class Grid(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int * 3), ("origin", ctypes.c_float * 3),
                ("spacing", ctypes.c_float * 3)]


class Beam(ctypes.Structure):
    _fields_ = [("src", ctypes.c_double * 3), ("vy", ctypes.c_double * 3),
                ("xform", ctypes.c_double * 9), ("sad", ctypes.c_double),
                ("geom_f32", ctypes.c_int), ("sad_f32", ctypes.c_int),
                ("block", ctypes.c_void_p), ("block_rows", ctypes.c_int),
                ("block_cols", ctypes.c_int), ("block_r0", ctypes.c_int),
                ("block_c0", ctypes.c_int), ("full_rows", ctypes.c_int),
                ("full_cols", ctypes.c_int), ("block_uniform", ctypes.c_int)]


SETTING_KEYS = ("sPri", "sAnn", "zAnn", "rInner", "rOuter", "zExp", "sExp", "kExp",
                "softRatio", "softLimit", "hornRatio")


class Settings(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in SETTING_KEYS] + [
        ("samples", ctypes.c_int), ("n_energy", ctypes.c_int),
        ("E", ctypes.c_float * CH_MAX_ENERGY), ("w", ctypes.c_float * CH_MAX_ENERGY),
        ("mu", ctypes.c_float * CH_MAX_ENERGY), ("options", ctypes.c_int)]


CH_OPT_RADIOLOGICAL_DISTANCE = 1
CH_OPT_CONES_IN_BEAM_FRAME = 2


class Kernel(ctypes.Structure):
    _fields_ = [("n_phi", ctypes.c_int), ("n_r", ctypes.c_int), ("n_theta", ctypes.c_int),
                ("cum", ctypes.c_void_p), ("theta", ctypes.c_void_p), ("phi", ctypes.c_void_p)]


class Intermediates(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in
                ("blocked", "d_eff", "oad", "fluence", "f_soften", "f_horn", "terma")]


class MLC(ctypes.Structure):
    _fields_ = [("n_pairs", ctypes.c_int), ("map_rows", ctypes.c_int), ("map_cols", ctypes.c_int),
                ("open_r0", ctypes.c_int), ("open_r1", ctypes.c_int), ("open_c0", ctypes.c_int),
                ("open_c1", ctypes.c_int), ("reserved", ctypes.c_int),
                ("row0", ctypes.c_int * CH_MAX_LEAF_PAIRS), ("rows", ctypes.c_int * CH_MAX_LEAF_PAIRS),
                ("a_end", ctypes.c_int * CH_MAX_LEAF_PAIRS), ("b_start", ctypes.c_int * CH_MAX_LEAF_PAIRS),
                ("tip", ctypes.c_double * CH_MLC_TIP_CELLS)]


class Beamlets(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int), ("cols", ctypes.c_int), ("cell_rows", ctypes.c_int),
                ("cell_cols", ctypes.c_int), ("r0", ctypes.c_int), ("c0", ctypes.c_int)]


class Tuning(ctypes.Structure):
    _fields_ = [("dir_group", ctypes.c_int), ("unit_order", ctypes.c_int), ("terma_ctas_per_sm", ctypes.c_int),
                ("cone_method", ctypes.c_int)]


CONE_SPECTRAL, CONE_GATHER = 0, 1     # ch_tuning.cone_method


class Stats(ctypes.Structure):
    _fields_ = [("ms_prologue", ctypes.c_float), ("ms_range", ctypes.c_float),
                ("ms_cone", ctypes.c_float), ("updates", ctypes.c_double),
                ("n_unique_dirs", ctypes.c_int), ("n_units", ctypes.c_int)]


# name -> (restype, argtypes); every symbol the header declares
P = ctypes.POINTER
VP = ctypes.c_void_p
SIGNATURES = {
    "ch_plan_create": (ctypes.c_int, [P(VP), ctypes.c_int]),
    "ch_plan_destroy": (None, [VP]),
    "ch_plan_set_kernel": (ctypes.c_int, [VP, P(Kernel)]),
    "ch_dose": (ctypes.c_int, [VP, P(Grid), VP, ctypes.c_int, P(Beam), P(Settings), VP, VP]),
    "ch_dose_ex": (ctypes.c_int, [VP, P(Grid), VP, ctypes.c_int, P(Beam), P(Settings), VP,
                                  P(Intermediates), VP]),
    "ch_dose_batch": (ctypes.c_int, [VP, ctypes.c_int, P(Grid), P(VP), P(ctypes.c_int), P(Beam),
                                     P(Settings), P(VP), VP]),
    "ch_dose_scatter": (ctypes.c_int, [VP, P(Grid), VP, ctypes.c_int, P(Beam), P(Settings), VP, VP]),
    "ch_dose_static": (ctypes.c_int, [VP, P(Grid), VP, ctypes.c_int, P(Beam), P(Settings), VP, VP]),
    "ch_block_from_mlc": (ctypes.c_int, [P(MLC), VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         VP]),
    "ch_block_from_beamlets": (ctypes.c_int, [P(Beamlets), VP, VP, VP]),
    "ch_cone": (ctypes.c_int, [VP, P(Grid), VP, VP, ctypes.c_int, VP]),
    "ch_dose_adjoint": (ctypes.c_int, [VP, P(Grid), VP, ctypes.c_int, P(Beam), P(Beamlets), P(Settings), VP, VP, VP,
                                       VP]),
    "ch_dda_trace": (ctypes.c_int, [P(Grid), ctypes.c_int, VP, VP, ctypes.c_int, VP, VP, VP, VP]),
    "ch_cone_directions": (ctypes.c_int, [VP, VP, VP]),
    "ch_plan_set_tuning": (ctypes.c_int, [VP, P(Tuning)]),
    "ch_plan_get_tuning": (ctypes.c_int, [VP, P(Tuning)]),
    "ch_batch_create": (ctypes.c_int, [VP, ctypes.c_int, P(Grid), P(VP), P(ctypes.c_int), P(Beam), P(Settings),
                                       P(VP), VP, P(VP)]),
    "ch_batch_launch": (ctypes.c_int, [VP, VP]),
    "ch_batch_sync": (ctypes.c_int, [VP, VP]),
    "ch_batch_destroy": (None, [VP]),
    "ch_plan_prepare": (ctypes.c_int, [VP, P(Grid), VP]),
    "ch_plan_memory": (ctypes.c_int, [VP, P(ctypes.c_size_t), P(ctypes.c_size_t)]),
    "ch_batch_scratch_bytes": (ctypes.c_int, [VP, ctypes.c_int, P(Grid), P(ctypes.c_size_t),
                                              P(ctypes.c_size_t)]),
    "ch_plan_trim": (ctypes.c_int, [VP]),
    "ch_plan_sync": (ctypes.c_int, [VP, VP]),
    "ch_plan_set_wait_limit": (ctypes.c_int, [VP, ctypes.c_longlong, ctypes.c_int]),
    "ch_plan_stats": (ctypes.c_int, [VP, P(Stats)]),
    "ch_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "ch_last_error": (ctypes.c_char_p, []),
    "ch_version": (ctypes.c_int, []),
}

_lib = None


def library_path():
    return LIB


def lib():
    """Load the CUDA library (raises if it was never built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(
                f"conehead_gb300 CUDA library not found at {LIB}; run "
                "`python -m conehead_gb300.build` (there is no CPU fallback)")
        L = ctypes.CDLL(LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class CHError(RuntimeError):
    def __init__(self, status, where):
        msg = lib().ch_last_error().decode(errors="replace")
        super().__init__(f"{where}: {STATUS.get(status, status)}: {msg}")
        self.status = status


def check(status, where):
    if status != 0:
        if status == 5:
            raise RuntimeError("no intersection or line is within plane")
        raise CHError(status, where)


# -------------------------------------------------------------- helpers --
def grid_struct(size, origin, spacing):
    g = Grid()
    for k in range(3):
        g.n[k] = int(size[k])
        g.origin[k] = float(np.float32(origin[k]))
        g.spacing[k] = float(np.float32(spacing[k]))
    return g


def settings_struct(settings):
    from .nist import mu_water
    s = Settings()
    for k in SETTING_KEYS:
        setattr(s, k, float(settings[k]))
    s.samples = int(settings["fluenceResampling"])
    ew = settings["energy_weights"]
    if len(ew) > CH_MAX_ENERGY:
        raise ValueError(f"at most {CH_MAX_ENERGY} spectrum bins")
    E = np.array([np.float32(x) for x in ew.keys()], dtype=np.float32)
    w = np.array([np.float32(x) for x in ew.values()], dtype=np.float32)
    mu = np.asarray(mu_water(E), dtype=np.float32)
    s.n_energy = len(E)
    for i in range(len(E)):
        s.E[i] = float(E[i])
        s.w[i] = float(w[i])
        s.mu[i] = float(mu[i])
    s.options = physics_options(settings)
    return s


def physics_options(settings):
    """CH_OPT_* bits from the extension keys of a settings dict (absent in the
    reference's dicts, so reference settings give 0):
    "coneDistance": "geometric" (default) | "radiological";
    "coneFrame": "room" (default) | "beam"."""
    opts = 0
    dist = settings.get("coneDistance", "geometric")
    if dist not in ("geometric", "radiological"):
        raise ValueError(f"coneDistance must be 'geometric' or 'radiological', not {dist!r}")
    if dist == "radiological":
        opts |= CH_OPT_RADIOLOGICAL_DISTANCE
    frame = settings.get("coneFrame", "room")
    if frame not in ("room", "beam"):
        raise ValueError(f"coneFrame must be 'room' or 'beam', not {frame!r}")
    if frame == "beam":
        opts |= CH_OPT_CONES_IN_BEAM_FRAME
    return opts


def block_crop(block_values):
    """(crop float32 array, r0, c0): smallest box holding every nonzero value."""
    bv = np.asarray(block_values, dtype=np.float32)
    rows = np.flatnonzero(bv.any(axis=1))
    if rows.size == 0:
        return np.zeros((1, 1), dtype=np.float32), 0, 0
    cols = np.flatnonzero(bv[rows[0]:rows[-1] + 1].any(axis=0))
    r0, r1, c0, c1 = rows[0], rows[-1] + 1, cols[0], cols[-1] + 1
    return np.ascontiguousarray(bv[r0:r1, c0:c1]), int(r0), int(c0)


def beam_struct(source, block_dev_ptr, crop_shape, r0, c0, full_shape, uniform=False):
    b = Beam()
    pos = np.asarray(source.position)
    vy = np.asarray(source.v_y)
    xf = np.asarray(source.transform)
    b.geom_f32 = int(pos.dtype == np.float32 and vy.dtype == np.float32 and xf.dtype == np.float32)
    b.sad_f32 = int(isinstance(source.sad, np.float32))
    for k in range(3):
        b.src[k] = float(pos[k])
        b.vy[k] = float(vy[k])
    flat = xf.reshape(-1)
    for k in range(9):
        b.xform[k] = float(flat[k])
    b.sad = float(source.sad)
    b.block = block_dev_ptr
    b.block_rows, b.block_cols = int(crop_shape[0]), int(crop_shape[1])
    b.block_r0, b.block_c0 = int(r0), int(c0)
    b.full_rows, b.full_cols = int(full_shape[0]), int(full_shape[1])
    b.block_uniform = int(bool(uniform))
    return b
