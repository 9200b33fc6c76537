"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run once in a container that has the conehead sources (read-only), named
by ``--ref`` or by the environment variable ``CONEHEAD_REFERENCE``::

    python tests/golden/make_golden.py --ref /path/to/conehead

Three fixture families:

1. ``pipeline_<case>.npz`` -- the reference's own ``Conehead.calculate``
   (conehead/conehead.py:522-738) executed on small grids.  Numba is not
   installable here, so the ``@cuda.jit`` kernels run under a stand-in
   launcher (every thread of the grid called in turn, like Numba's own
   CUDA simulator) that reproduces Numba's scalar typing where plain
   NumPy would differ:
     * Python float / int kernel arguments become float64 / int64 scalars
       (Numba types them so);
     * ``cuda.grid`` returns int64 indices;
     * ``math.sqrt`` / ``math.exp`` of a float32 return float32 and
       ``math.pi`` is a float64 scalar (Numba's math typing);
     * the few float32 local arrays that Numba reads inside a float64
       expression (the hit-test ``position``/``offset`` arrays and the
       cone kernel's t-value array) are read back as float64.
   The reference's matplotlib/pydicom imports are stubbed; plotting is cut
   off before it starts.  Captured: blocked, d_eff, oad, fluence,
   f_soften, f_horn, TERMA and dose, plus every input.
2. ``dda_ref.npz`` -- voxel/t-value traces from conehead's compiled Cython
   ``dda_3d_c`` (oracle/build_ref.py) for a battery of directions/grids,
   including the notebook cases (dir (1,2,3)/sqrt(14) from (50,50,50) of
   101^3; dir (0.997859, 0, -0.065403) on 41^3).
4. ``plans.npz`` -- ``Block(plan=...)`` (conehead/block.py:87-215) run on
   the reference's RT Plan fixture (RP.3DCRT.dcm, read with this package's
   pydicom-free reader) and on seeded synthetic plans (Millennium-,
   Agility- and HD120-like leaf banks, colliding leaves, jaws beyond the map,
   a two-beam plan): every input number, the SHA-256 of each full map and
   the map inside its nonzero bounding box, or the error the reference
   raises (maps other than 4000 rows).
3. ``tables.npz`` -- the reference's host tables: ``KernelPoly.kernel_cum``
   for the example.py spectrum (every 7th column plus the last, and the
   full row sums), the 48 cone angles, ``mu_water`` at the
   twelve spectrum energies, Source geometry at several gantry/collimator
   angles and ``Block.set_square`` bounds.
"""
import argparse
import math as _math
import multiprocessing as mp
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))

EXAMPLE_SETTINGS = {
    'sPri': 0.90924, 'sAnn': 2.887e-3, 'zAnn': 4.0, 'rInner': 0.2, 'rOuter': 1.4,
    'zExp': 12.5, 'sExp': 8.289e-3, 'kExp': 0.4816, 'softRatio': 0.0025,
    'softLimit': 20, 'hornRatio': 0.0065, 'fluenceResampling': 3,
    'energy_weights': {"0.5": 0.08196, "1.0": 0.12385, "1.5": 0.10605, "2.0": 0.08307,
                       "2.5": 0.05881, "3.0": 0.03911, "3.5": 0.02131, "4.0": 0.02426,
                       "4.5": 0.0, "5.0": 0.00881, "5.5": 0.0, "6.0": 0.00498},
}

# (name, size, origin, spacing, gantry, collimator, square_cm, density seed)
# gantry None = fresh Source (float32 geometry arrays)
CASES = [
    ("g0_water_slab", (10, 10, 10), (-2.25, 0.25, -2.25), (0.5, 0.5, 0.5), 0.0, 0.0, 3.0, None),
    ("oblique_hetero", (10, 10, 10), (-1.8, -1.8, -1.8), (0.4, 0.4, 0.4), 30.0, 20.0, 2.0, 7),
    ("aniso_f32geom", (9, 9, 7), (-1.6, 0.3, -0.9), (0.4, 0.5, 0.3), None, None, 2.0, 11),
]


# ---------------------------------------------------------------- stand-in
class _F64Read(np.ndarray):
    """float32 storage whose scalar reads come back as float64."""

    def __getitem__(self, key):
        v = np.ndarray.__getitem__(self, key)
        if isinstance(v, np.floating):
            return np.float64(v)
        return v


class _DeviceArray(np.ndarray):
    def copy_to_host(self):
        out = np.array(self)
        _EVENTS.append(("d2h", out))
        return out


_EVENTS = []
_THREAD = [0, 0, 0]
_ALLOC = {"count": 0}


class _StopCalc(Exception):
    pass


def _install_stubs():
    numba = types.ModuleType("numba")
    numba.float32 = np.float32
    numba.float64 = np.float64
    numba.int32 = np.int32
    cuda = types.ModuleType("numba.cuda")

    def to_device(a):
        arr = np.array(a)
        _EVENTS.append(("h2d", arr))
        return arr.view(_DeviceArray)

    def grid(n):
        return tuple(np.int64(v) for v in _THREAD[:n])

    def local_array(shape, dtype):
        caller = sys._getframe(1).f_code.co_name
        arr = np.zeros(shape, dtype=dtype)
        if caller == "cuda_hit_test":
            _ALLOC["count"] += 1
            if _ALLOC["count"] <= 2:          # `position`, `offset`
                return arr.view(_F64Read)
        if caller == "cuda_dose" and dtype is np.float32 and shape == 800:
            return arr.view(_F64Read)         # intersection_t_values
        return arr

    def atomic_add(arr, idx, val):
        arr[idx] = arr[idx] + arr.dtype.type(val)

    class _Kernel:
        def __init__(self, fn):
            self.fn = fn

        def __getitem__(self, cfg):
            blocks, threads = cfg
            dims = [int(b) * int(t) for b, t in zip(blocks, threads)]
            fn = self.fn

            def launch(*args):
                conv = []
                for a in args:
                    if type(a) is float:
                        conv.append(np.float64(a))
                    elif type(a) is int:
                        conv.append(np.int64(a))
                    else:
                        conv.append(a)
                for x in range(dims[0]):
                    for y in range(dims[1]):
                        for z in range(dims[2]):
                            _THREAD[:] = [x, y, z]
                            _ALLOC["count"] = 0
                            fn(*conv)
            return launch

    def jit(fn=None, device=False, **kw):
        if fn is None:
            return lambda f: jit(f, device=device)
        return fn if device else _Kernel(fn)

    cuda.jit = jit
    cuda.to_device = to_device
    cuda.grid = grid
    cuda.local = types.SimpleNamespace(array=local_array)
    cuda.atomic = types.SimpleNamespace(add=atomic_add)
    numba.cuda = cuda
    sys.modules["numba"] = numba
    sys.modules["numba.cuda"] = cuda

    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")

    def subplots(*a, **k):
        raise _StopCalc()
    plt.subplots = subplots
    mpl.pyplot = plt
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt

    pyd = types.ModuleType("pydicom")
    pyd_ds = types.ModuleType("pydicom.dataset")
    pyd_ds.FileDataset = object
    pyd.dataset = pyd_ds
    sys.modules["pydicom"] = pyd
    sys.modules["pydicom.dataset"] = pyd_ds


def _numba_math():
    """``math`` as Numba types it for float32 arguments."""
    m = types.SimpleNamespace(**{k: getattr(_math, k) for k in dir(_math)
                                 if not k.startswith("_")})
    m.pi = np.float64(_math.pi)
    m.sqrt = lambda x: np.float32(np.sqrt(x)) if isinstance(x, np.float32) else _math.sqrt(x)
    m.exp = lambda x: np.float32(np.exp(x)) if isinstance(x, np.float32) else _math.exp(x)
    m.pow = lambda x, y: _math.pow(float(x), float(y))
    return m


def _run_case(args):
    case, ref = args
    name, size, origin, spacing, gantry, collim, square, seed = case
    _install_stubs()
    sys.path.insert(0, ref)
    import conehead.conehead as ch
    from conehead.source import Source
    from conehead.block import Block
    ch.math = _numba_math()
    n = list(size)
    if seed is None:
        rho = np.ones(n, dtype=np.float32)
        rho[:, n[1] // 2:n[1] // 2 + 2, :] = 1.6
    else:
        rho = np.random.default_rng(seed).uniform(0.2, 2.0, n).astype(np.float32)
    phantom = types.SimpleNamespace(size=n, origin=np.array(origin, dtype=np.float32),
                                    spacing=np.array(spacing, dtype=np.float32),
                                    densities=rho)
    source = Source("varian_clinac_6MV")
    if gantry is not None:
        source.gantry = gantry
        source.collimator = collim
    block = Block()
    block.set_square(square)
    cwd = os.getcwd()
    os.chdir(ref)
    _EVENTS.clear()
    try:
        ch.Conehead().calculate(source, block, phantom, dict(EXAMPLE_SETTINGS))
    except _StopCalc:
        pass
    finally:
        os.chdir(cwd)
    d2h = [a for kind, a in _EVENTS if kind == "d2h"]
    blocked, d_eff, oad, fluence, terma, dose = d2h
    # f_soften / f_horn: the two host arrays uploaded right after the fluence D2H
    idx = [i for i, (k, a) in enumerate(_EVENTS) if k == "d2h"][3]
    later = [a for k, a in _EVENTS[idx + 1:] if k == "h2d"]
    f_soften, f_horn = later[0], later[1]
    out = dict(size=np.array(n), origin=phantom.origin, spacing=phantom.spacing,
               densities=rho, gantry=np.float64(-1 if gantry is None else gantry),
               collimator=np.float64(-1 if collim is None else collim),
               square=np.float64(square), position=np.asarray(source.position),
               v_y=np.asarray(source.v_y), transform=np.asarray(source.transform),
               sad=np.asarray(source.sad), blocked=blocked, d_eff=d_eff, oad=oad,
               fluence=fluence, f_soften=f_soften, f_horn=f_horn, terma=terma, dose=dose)
    path = os.path.join(HERE, f"pipeline_{name}.npz")
    np.savez_compressed(path, **out)
    return path


def make_dda(ref):
    sys.path.insert(0, REPO)
    from oracle import build_ref
    build_ref.build(ref)
    shim = build_ref.load()
    rng = np.random.default_rng(2024)
    traces = []
    # notebook known-answer cases (dda_benchmarking.ipynb cells 3/10 and 14-16)
    nb = [((1 / 14 ** .5, 2 / 14 ** .5, 3 / 14 ** .5), (101, 101, 101), (50, 50, 50), (1., 1., 1.)),
          ((0.997859, 0.0, -0.065403), (41, 41, 41), (20, 20, 20), (1., 1., 1.))]
    for c in nb:
        traces.append(c)
    for _ in range(300):
        d = rng.normal(size=3)
        if rng.random() < 0.2:
            d[rng.integers(3)] = 0.0
        d = d / np.linalg.norm(d)
        n = tuple(int(v) for v in rng.integers(5, 48, size=3))
        s = tuple(int(rng.integers(0, v)) for v in n)
        sp = tuple(float(np.float32(v)) for v in rng.choice([0.1, 0.2, 0.25, 0.3, 0.5, 1.0], size=3))
        traces.append((tuple(d), n, s, sp))
    dirs, shapes, starts, spacings, offs, vox, tv = [], [], [], [], [0], [], []
    for d, n, s, sp in traces:
        v, t = shim.trace(d, n, s, sp)
        dirs.append(d)
        shapes.append(n)
        starts.append(s)
        spacings.append(sp)
        vox.extend(v)
        tv.extend(t)
        offs.append(len(tv))
    np.savez_compressed(os.path.join(HERE, "dda_ref.npz"), direction=np.array(dirs),
                        shape=np.array(shapes, dtype=np.int32),
                        start=np.array(starts, dtype=np.int32),
                        spacing=np.array(spacings, dtype=np.float64),
                        offsets=np.array(offs, dtype=np.int64),
                        voxels=np.array(vox, dtype=np.int32).reshape(-1, 3),
                        tvals=np.array(tv, dtype=np.float64))


def make_tables(ref):
    sys.path.insert(0, ref)
    _install_stubs()
    from conehead.kernel import KernelMono, KernelPoly
    from conehead.nist import mu_water
    from conehead.source import Source
    from conehead.block import Block
    cwd = os.getcwd()
    os.chdir(ref)
    try:
        files = {"0.5": "0.5", "1.0": "1.5", "1.5": "1.5", "2.0": "2.0", "2.5": "2.5",
                 "3.0": "3.0", "3.5": "3.5", "4.0": "4.0", "4.5": "4.5", "5.0": "5.0",
                 "5.5": "5.5", "6.0": "6.0"}
        kernels = {e: KernelMono(f"kernels/{f}MeV/{f}MeV.egslst") for e, f in files.items()}
    finally:
        os.chdir(cwd)
    ew = EXAMPLE_SETTINGS["energy_weights"]
    kd = np.zeros_like(kernels["0.5"].kernel_diff)
    for e in ew:
        kd += kernels[e].kernel_diff * ew[e]
    kd = kd / kd.sum()
    poly = KernelPoly(kernels["0.5"].angles, kernels["0.5"].radii, kd)
    E = np.array([np.float32(x) for x in ew.keys()], dtype=np.float32)
    geo = []
    for g, c in [(0, 0), (45, 0), (225, 0), (270, 0), (0, 90), (0, 270), (315, 45), (37.5, 12.25), (183, 77)]:
        s = Source("varian_clinac_6MV")
        s.gantry = g
        s.collimator = c
        geo.append(np.concatenate([[g, c], s.position, s.v_y, np.asarray(s.transform).ravel()]))
    sq = []
    for L in (1.0, 2.5, 3.0, 5.0, 10.0, 12.3, 40.0):
        b = Block()
        b.set_square(L)
        nz = np.argwhere(b.block_values > 0)
        sq.append([L, nz[:, 0].min(), nz[:, 0].max(), nz[:, 1].min(), nz[:, 1].max(), b.block_values.sum()])
    cols = np.r_[0:poly.kernel_cum.shape[1]:7, poly.kernel_cum.shape[1] - 1]
    np.savez_compressed(os.path.join(HERE, "tables.npz"), kernel_cum_cols=cols,
                        kernel_cum_sub=poly.kernel_cum[:, cols],
                        kernel_cum_rowsum=poly.kernel_cum.sum(axis=1),
                        phis=poly.angles, energies=E, mu_water=mu_water(E),
                        mu_water_2MeV=np.float64(mu_water(2.0)),
                        geometry=np.array(geo), squares=np.array(sq, dtype=np.float64))


def _plan_ns(beams):
    """An RT Plan as nested namespaces with the keywords Block reads."""
    ns = types.SimpleNamespace
    out = []
    for bm in beams:
        devs = [ns(RTBeamLimitingDeviceType=t, LeafPositionBoundaries=list(map(float, b)))
                for t, b in bm["devices"]]
        pos = [ns(RTBeamLimitingDeviceType=t, LeafJawPositions=list(map(float, v)))
               for t, v in bm["positions"]]
        out.append(ns(BeamType=bm.get("type", "STATIC"), BeamLimitingDeviceSequence=devs,
                      ControlPointSequence=[ns(BeamLimitingDevicePositionSequence=pos)]))
    return ns(BeamSequence=out)


def synthetic_plans(seed=5):
    """Seeded plan descriptions (dicts of plain numbers)."""
    rng = np.random.default_rng(seed)
    plans = {}
    # Millennium-120-like bank: 10 mm outer, 5 mm inner leaves over +-200 mm
    mil = np.r_[np.arange(-200, -100, 10), np.arange(-100, 100, 5), np.arange(100, 201, 10)].astype(float)
    n = len(mil) - 1
    a = rng.uniform(-90, 30, n).round(1)
    b = (a + rng.uniform(0.5, 80, n)).round(1)
    plans["millennium_random"] = [dict(devices=[("MLCX", mil)], positions=[
        ("ASYMX", [-61.3, 47.8]), ("ASYMY", [-73.0, 55.5]), ("MLCX", np.r_[a, b])])]
    # Agility-like: 80 pairs of 5 mm; some leaves colliding (A beyond B)
    agi = np.arange(-200, 201, 5).astype(float)
    n = len(agi) - 1
    a = rng.uniform(-60, 40, n).round(2)
    b = a + rng.uniform(-6, 50, n).round(2)
    plans["agility_collide"] = [dict(devices=[("MLCX", agi)], positions=[
        ("X", [-45.0, 45.0]), ("Y", [-52.25, 38.75]), ("MLCX", np.r_[a, b])])]
    # HD120-like: map of 2200 rows (narrower than the 4000-cell lookup range)
    hd = np.r_[np.arange(-110, -40, 5), np.arange(-40, 40, 2.5), np.arange(40, 111, 5)].astype(float)
    n = len(hd) - 1
    a = rng.uniform(-30, 10, n).round(1)
    b = (a + rng.uniform(2, 40, n)).round(1)
    plans["hd120_narrow"] = [dict(devices=[("MLCX", hd)], positions=[
        ("ASYMX", [-25.0, 31.0]), ("ASYMY", [-48.0, 52.0]), ("MLCX", np.r_[a, b])])]
    # irregular boundaries (0.01 mm values) over the 400 mm span, jaws past
    # the map on the left and a crossed Y jaw: numpy's slice rules on
    # negative indices decide which rows and columns stay open
    w = rng.uniform(0.5, 1.0, 60)
    irr = np.r_[-200.0, (-200.0 + np.cumsum(w / w.sum() * 400.0))[:-1].round(2), 200.0]
    n = len(irr) - 1
    a = rng.uniform(-50, 20, n).round(1)
    b = (a + rng.uniform(1, 60, n)).round(1)
    plans["irregular_wide_jaws"] = [dict(devices=[("MLCX", irr)], positions=[
        ("ASYMX", [-250.0, 210.0]), ("ASYMY", [-150.0, -230.0]), ("MLCX", np.r_[a, b])])]
    # two beams: the second control point has no X jaw, so the first beam's
    # X jaw stays in force (the reference keeps the last value it read)
    a1 = np.full(60, -20.0)
    b1 = np.full(60, 20.0)
    a2 = rng.uniform(-40, 0, 60).round(1)
    b2 = (a2 + rng.uniform(5, 50, 60)).round(1)
    plans["two_beams"] = [
        dict(devices=[("ASYMX", [0.0]), ("MLCX", mil)], positions=[
            ("ASYMX", [-30.0, 30.0]), ("ASYMY", [-30.0, 30.0]), ("MLCX", np.r_[a1, b1])]),
        dict(devices=[("MLCX", mil)], positions=[
            ("ASYMY", [-44.0, 36.0]), ("MLCX", np.r_[a2, b2])])]
    return plans


def make_plans(ref):
    sys.path.insert(0, ref)
    sys.path.insert(0, REPO)
    _install_stubs()
    import hashlib
    from conehead.block import Block as RefBlock
    from conehead_gb300 import dicom
    out = {}
    cases = {"fixture": dicom.read(os.path.join(ref, "RP.3DCRT.dcm"), force=True)}
    descs = synthetic_plans()
    for name, d in descs.items():
        cases[name] = _plan_ns(d)
        for i, bm in enumerate(d):
            for j, (t, v) in enumerate(bm["devices"]):
                out[f"{name}/beam{i}/dev{j}/{t}"] = np.asarray(v, dtype=np.float64)
            for j, (t, v) in enumerate(bm["positions"]):
                out[f"{name}/beam{i}/pos{j}/{t}"] = np.asarray(v, dtype=np.float64)
    for name, plan in cases.items():
        try:
            bv = RefBlock(plan=plan).block_values
        except ValueError as e:          # maps that are not 4000 rows (scipy interpolator check)
            out[f"{name}/raises"] = np.array(str(e))
            continue
        assert bv.dtype == np.float32
        nz = np.argwhere(bv != 0)
        r0, c0 = nz.min(axis=0)
        r1, c1 = nz.max(axis=0) + 1
        out[f"{name}/shape"] = np.array(bv.shape)
        out[f"{name}/sha256"] = np.frombuffer(hashlib.sha256(bv.tobytes()).digest(), dtype=np.uint8)
        out[f"{name}/bbox"] = np.array([r0, r1, c0, c1])
        out[f"{name}/crop"] = bv[r0:r1, c0:c1]
    np.savez_compressed(os.path.join(HERE, "plans.npz"), **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CONEHEAD_REFERENCE"),
                    help="conehead checkout (default: $CONEHEAD_REFERENCE)")
    ap.add_argument("--only", default=None, help="pipeline|dda|tables|plans")
    a = ap.parse_args()
    if not a.ref:
        ap.error("name the conehead checkout with --ref or CONEHEAD_REFERENCE")
    if a.only in (None, "tables"):
        make_tables(a.ref)
        print("tables done")
    if a.only in (None, "plans"):
        make_plans(a.ref)
        print("plans done")
    if a.only in (None, "dda"):
        make_dda(a.ref)
        print("dda done")
    if a.only in (None, "pipeline"):
        with mp.get_context("spawn").Pool(len(CASES)) as pool:
            for p in pool.imap_unordered(_run_case, [(c, a.ref) for c in CASES]):
                print("wrote", p)


if __name__ == "__main__":
    main()
