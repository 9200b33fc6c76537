"""Python front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Wraps ``oracle/_build/liboracle.so`` (built from ``oracle/oracle.cpp`` by
``oracle/Makefile``) with a ``calculate`` that mirrors the reference's
``Conehead.calculate`` (conehead/conehead.py:522-738) step for step and
returns every intermediate.  Only tests, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg use it; the engine never does.

Host-side tables (the EDKnrc cumulative kernel and ``mu_water``) come from
``conehead_gb300.kernel`` / ``conehead_gb300.nist``; those two modules are
pinned bit-for-bit against the reference's own ``kernel.py``/``nist.py``
output by the golden fixtures in tests/golden.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

MODE_F32 = 0   # float32-mirrored (Numba typing of the reference kernels)
MODE_F64 = 1   # FP64 re-run of the same algorithm

SETTING_KEYS = ("sPri", "sAnn", "zAnn", "rInner", "rOuter", "zExp", "sExp",
                "kExp", "softRatio", "softLimit", "hornRatio")


class _Grid(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int * 3), ("origin", ctypes.c_float * 3),
                ("spacing", ctypes.c_float * 3)]


class _Beam(ctypes.Structure):
    _fields_ = [("src", ctypes.c_double * 3), ("vy", ctypes.c_double * 3),
                ("xform", ctypes.c_double * 9), ("sad", ctypes.c_double),
                ("geom_f32", ctypes.c_int), ("sad_f32", ctypes.c_int),
                ("block", ctypes.POINTER(ctypes.c_float)),
                ("block_rows", ctypes.c_int), ("block_cols", ctypes.c_int)]


class _Settings(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in SETTING_KEYS] + [
        ("samples", ctypes.c_int), ("n_energy", ctypes.c_int),
        ("E", ctypes.POINTER(ctypes.c_float)), ("w", ctypes.POINTER(ctypes.c_float)),
        ("mu", ctypes.POINTER(ctypes.c_float))]


_lib = None


def build():
    """Compile the oracle library (no-op when up to date)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        dp = P(ctypes.c_double)
        L.or_prologue.argtypes = [P(_Grid), P(ctypes.c_float), ctypes.c_int, P(_Beam),
                                  P(_Settings), ctypes.c_int] + [dp] * 7
        L.or_prologue.restype = ctypes.c_int
        L.or_cone.argtypes = [P(_Grid), dp, dp, ctypes.c_int, P(ctypes.c_float), ctypes.c_int,
                              P(ctypes.c_float), ctypes.c_int, ctypes.c_int, dp]
        L.or_cone.restype = None
        L.or_cone_ext.argtypes = [P(_Grid), dp, dp, ctypes.c_int, P(ctypes.c_float), ctypes.c_int,
                                  P(ctypes.c_float), ctypes.c_int, ctypes.c_int, P(ctypes.c_float), ctypes.c_int,
                                  dp, dp]
        L.or_cone_ext.restype = None
        L.or_cone_transpose.argtypes = L.or_cone.argtypes
        L.or_cone_transpose.restype = None
        L.or_cone_transpose_on.argtypes = L.or_cone.argtypes[:-1] + [dp, dp]
        L.or_cone_transpose_on.restype = None
        L.or_blocked_adjoint.argtypes = [P(_Grid), P(_Beam), ctypes.c_int, dp] + [ctypes.c_int] * 6 + [dp]
        L.or_blocked_adjoint.restype = ctypes.c_int
        L.or_dda.argtypes = [P(ctypes.c_int), P(ctypes.c_float), P(ctypes.c_int), dp,
                             ctypes.c_int, ctypes.c_int, P(ctypes.c_int), dp]
        L.or_dda.restype = ctypes.c_int
        L.or_cone_direction.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int, dp]
        L.or_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def num_threads():
    return lib().or_num_threads()


def grid_struct(size, origin, spacing):
    g = _Grid()
    for k in range(3):
        g.n[k] = int(size[k])
        g.origin[k] = float(np.float32(origin[k]))
        g.spacing[k] = float(np.float32(spacing[k]))
    return g


def beam_struct(source, block_values):
    b = _Beam()
    pos = np.asarray(source.position)
    vy = np.asarray(source.v_y)
    xf = np.asarray(source.transform)
    b.geom_f32 = int(pos.dtype == np.float32 and vy.dtype == np.float32 and xf.dtype == np.float32)
    b.sad_f32 = int(isinstance(source.sad, np.float32))
    for k in range(3):
        b.src[k] = float(pos[k])
        b.vy[k] = float(vy[k])
    for k in range(9):
        b.xform[k] = float(xf.reshape(-1)[k])
    b.sad = float(source.sad)
    b.block = _ptr(block_values, ctypes.c_float)
    b.block_rows, b.block_cols = block_values.shape
    return b


def settings_struct(settings, E, w, mu):
    s = _Settings()
    for k in SETTING_KEYS:
        setattr(s, k, float(settings[k]))
    s.samples = int(settings["fluenceResampling"])
    s.n_energy = len(E)
    s.E = _ptr(E, ctypes.c_float)
    s.w = _ptr(w, ctypes.c_float)
    s.mu = _ptr(mu, ctypes.c_float)
    return s


def spectrum(settings):
    from conehead_gb300.nist import mu_water
    ew = settings["energy_weights"]
    E = np.array([np.float32(x) for x in ew.keys()], dtype=np.float32)
    w = np.array([np.float32(x) for x in ew.values()], dtype=np.float32)
    mu = np.ascontiguousarray(mu_water(E), dtype=np.float32)
    return E, w, mu


def prologue(source, block, phantom, settings, mode=MODE_F32, swap_xy=None):
    """Blocked, d_eff, oad, fluence, f_soften, f_horn and TERMA (float64 arrays)."""
    size = [int(n) for n in phantom.size]
    if swap_xy is None:
        swap_xy = size[0] == size[1]
    rho = np.ascontiguousarray(phantom.densities, dtype=np.float32)
    block_values = np.ascontiguousarray(block.block_values, dtype=np.float32)
    E, w, mu = spectrum(settings)
    g = grid_struct(size, phantom.origin, phantom.spacing)
    b = beam_struct(source, block_values)
    s = settings_struct(settings, E, w, mu)
    names = ("blocked", "d_eff", "oad", "fluence", "f_soften", "f_horn", "terma")
    out = {k: np.zeros(size, dtype=np.float64) for k in names}
    rc = lib().or_prologue(ctypes.byref(g), _ptr(rho, ctypes.c_float), int(swap_xy),
                           ctypes.byref(b), ctypes.byref(s), int(mode),
                           *[_ptr(out[k], ctypes.c_double) for k in names])
    if rc != 0:
        raise RuntimeError("no intersection or line is within plane")
    return out


def cone(terma, size, spacing, K, thetas, phis, mode=MODE_F32):
    """Collapsed-cone scatter of a TERMA grid; returns float64 dose."""
    size = [int(n) for n in size]
    T = np.ascontiguousarray(terma, dtype=np.float64)
    K = np.ascontiguousarray(K, dtype=np.float64)
    th = np.ascontiguousarray(thetas, dtype=np.float32)
    ph = np.ascontiguousarray(phis, dtype=np.float32)
    g = grid_struct(size, (0, 0, 0), spacing)
    dose = np.zeros(size, dtype=np.float64)
    lib().or_cone(ctypes.byref(g), _ptr(T, ctypes.c_double), _ptr(K, ctypes.c_double),
                  K.shape[1], _ptr(th, ctypes.c_float), len(th), _ptr(ph, ctypes.c_float),
                  len(ph), int(mode), _ptr(dose, ctypes.c_double))
    return dose


def cone_ext(terma, size, spacing, K, thetas, phis, mode=MODE_F32, rho=None, swap_xy=False, frame=None):
    """Cone stage with the physics extensions: ``rho`` (densities) for the
    radiological cone distance, ``frame`` (3x3 world->beam matrix) for cones
    in the beam frame."""
    size = [int(n) for n in size]
    T = np.ascontiguousarray(terma, dtype=np.float64)
    K = np.ascontiguousarray(K, dtype=np.float64)
    th = np.ascontiguousarray(thetas, dtype=np.float32)
    ph = np.ascontiguousarray(phis, dtype=np.float32)
    g = grid_struct(size, (0, 0, 0), spacing)
    dose = np.zeros(size, dtype=np.float64)
    r = None if rho is None else np.ascontiguousarray(rho, dtype=np.float32)
    f = None if frame is None else np.ascontiguousarray(np.asarray(frame, dtype=np.float64).reshape(9))
    lib().or_cone_ext(ctypes.byref(g), _ptr(T, ctypes.c_double), _ptr(K, ctypes.c_double), K.shape[1],
                      _ptr(th, ctypes.c_float), len(th), _ptr(ph, ctypes.c_float), len(ph), int(mode),
                      None if r is None else _ptr(r, ctypes.c_float), int(bool(swap_xy)),
                      None if f is None else _ptr(f, ctypes.c_double), _ptr(dose, ctypes.c_double))
    return dose


def cone_transpose(r, size, spacing, K, thetas, phis, mode=MODE_F64):
    """Transposed collapsed-cone stage of a dose-shaped grid; float64."""
    size = [int(n) for n in size]
    R = np.ascontiguousarray(r, dtype=np.float64)
    K = np.ascontiguousarray(K, dtype=np.float64)
    th = np.ascontiguousarray(thetas, dtype=np.float32)
    ph = np.ascontiguousarray(phis, dtype=np.float32)
    g = grid_struct(size, (0, 0, 0), spacing)
    out = np.zeros(size, dtype=np.float64)
    lib().or_cone_transpose(ctypes.byref(g), _ptr(R, ctypes.c_double), _ptr(K, ctypes.c_double),
                            K.shape[1], _ptr(th, ctypes.c_float), len(th), _ptr(ph, ctypes.c_float),
                            len(ph), int(mode), _ptr(out, ctypes.c_double))
    return out


def cone_transpose_on(r, support, size, spacing, K, thetas, phis, mode=MODE_F64):
    """Transposed cone of ``r`` computed only where ``support`` != 0 (0
    elsewhere); float64."""
    size = [int(n) for n in size]
    R = np.ascontiguousarray(r, dtype=np.float64)
    sup = np.ascontiguousarray(support, dtype=np.float64)
    K = np.ascontiguousarray(K, dtype=np.float64)
    th = np.ascontiguousarray(thetas, dtype=np.float32)
    ph = np.ascontiguousarray(phis, dtype=np.float32)
    g = grid_struct(size, (0, 0, 0), spacing)
    out = np.zeros(size, dtype=np.float64)
    lib().or_cone_transpose_on(ctypes.byref(g), _ptr(R, ctypes.c_double), _ptr(K, ctypes.c_double),
                               K.shape[1], _ptr(th, ctypes.c_float), len(th), _ptr(ph, ctypes.c_float),
                               len(ph), int(mode), _ptr(sup, ctypes.c_double), _ptr(out, ctypes.c_double))
    return out


def blocked_adjoint(source, block, phantom, settings, coef, beamlets):
    """Float64 transposed blocking onto a beamlet grid: grad[i, j] = sum over
    voxels v of coef[v] * (sub-samples of v whose block map cell lies in
    beamlet (i, j)) / S^3.  ``beamlets`` has rows, cols, cell_rows,
    cell_cols, r0 and c0 (map cells); ``block.block_values`` gives the map
    shape (the cell rule wraps index -1 to its last row / column)."""
    size = [int(n) for n in phantom.size]
    block_values = np.ascontiguousarray(block.block_values, dtype=np.float32)
    g = grid_struct(size, phantom.origin, phantom.spacing)
    b = beam_struct(source, block_values)
    c = np.ascontiguousarray(coef, dtype=np.float64)
    grad = np.zeros((beamlets.rows, beamlets.cols), dtype=np.float64)
    rc = lib().or_blocked_adjoint(ctypes.byref(g), ctypes.byref(b), int(settings["fluenceResampling"]),
                                  _ptr(c, ctypes.c_double), beamlets.rows, beamlets.cols, beamlets.cell_rows,
                                  beamlets.cell_cols, beamlets.r0, beamlets.c0, _ptr(grad, ctypes.c_double))
    if rc != 0:
        raise RuntimeError("no intersection or line is within plane")
    return grad


def beamlet_gradient_f64(source, beamlets, weights, phantom, settings, target, kernel_dir=None):
    """FP64 gradient of L = sum (dose - target)^2 with respect to beamlet
    weights, by the chain rule through the FP64 re-run of the reference path:
    the forward (prologue and cone), dL/dTERMA = C^T 2 (dose - target) on the
    TERMA support, and, since fluence and TERMA each carry one factor of the
    blocked fraction (conehead.py:360, :377), dTERMA/dblocked = 2 TERMA /
    blocked, pushed onto the beamlets by the transposed blocking.  Returns
    (grad [rows, cols], dose)."""
    from conehead_gb300.kernel import poly_kernel_tables

    class _Map:
        block_values = beamlets.host_map(weights)

    blk = _Map()
    out = prologue(source, blk, phantom, settings, MODE_F64)
    K, thetas, phis = poly_kernel_tables(settings["energy_weights"], kernel_dir)
    T, bl = out["terma"], out["blocked"]
    dose = cone(T, phantom.size, phantom.spacing, K, thetas, phis, MODE_F64)
    g_t = cone_transpose_on(2.0 * (dose - np.asarray(target, dtype=np.float64)), T, phantom.size, phantom.spacing,
                            K, thetas, phis, MODE_F64)
    coef = np.zeros_like(T)
    nz = bl > 0
    coef[nz] = 2.0 * g_t[nz] * T[nz] / bl[nz]
    return blocked_adjoint(source, blk, phantom, settings, coef, beamlets), dose


def calculate(source, block, phantom, settings, mode=MODE_F32, kernel_dir=None):
    """Full single-beam path; dict with the prologue outputs plus 'dose'."""
    from conehead_gb300.kernel import poly_kernel_tables
    out = prologue(source, block, phantom, settings, mode)
    K, thetas, phis = poly_kernel_tables(settings["energy_weights"], kernel_dir)
    out["dose"] = cone(out["terma"], phantom.size, phantom.spacing, K, thetas, phis, mode)
    return out


def dda(size, spacing, start, direction, mode=MODE_F32, cap=4096):
    """One DDA trace: (voxels int32 [L, 3], exit t-values float64 [L])."""
    n = np.ascontiguousarray(size, dtype=np.int32)
    sp = np.ascontiguousarray(spacing, dtype=np.float32)
    st = np.ascontiguousarray(start, dtype=np.int32)
    d = np.ascontiguousarray(direction, dtype=np.float64)
    vox = np.zeros((cap, 3), dtype=np.int32)
    tv = np.zeros(cap, dtype=np.float64)
    L = lib().or_dda(_ptr(n, ctypes.c_int), _ptr(sp, ctypes.c_float), _ptr(st, ctypes.c_int),
                     _ptr(d, ctypes.c_double), int(mode), cap, _ptr(vox, ctypes.c_int),
                     _ptr(tv, ctypes.c_double))
    L = min(L, cap)
    return vox[:L].copy(), tv[:L].copy()


def cone_direction(theta, phi, mode=MODE_F32):
    out = np.zeros(3, dtype=np.float64)
    lib().or_cone_direction(float(theta), float(phi), int(mode), _ptr(out, ctypes.c_double))
    return out
