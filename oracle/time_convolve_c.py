"""Time the reference's shipped Cython cone convolution -- a CPU datum.

conehead/convolve_c.pyx:14-274 is the reference's legacy CPU convolution,
compiled here from its unmodified sources (oracle/build_ref.py), single
threaded as shipped.  Its conventions differ from the live GPU path
(z-polar cone directions, kernel index floor(100 t - 50), no clamp), so it
is reported beside the engine's numbers as a datum, not compared with them.

Input: a TERMA field like the small plain-method case: 40^3 water at
0.5 cm, 10 x 10 cm field at gantry 0, TERMA from the FP64 oracle prologue;
the polyenergetic cumulative kernel of the example spectrum, 12 azimuths x
48 polar angles.  `tqdm` (a progress bar the module imports) is replaced by
a pass-through when it is not installed.  Prints one JSON line.

    python oracle/time_convolve_c.py
"""
import json
import os
import platform
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
for p in (REPO, os.path.join(HERE, "_ref")):
    if p not in sys.path:
        sys.path.insert(0, p)

SETTINGS = {
    'sPri': 0.90924, 'sAnn': 2.887e-3, 'zAnn': 4.0, 'rInner': 0.2, 'rOuter': 1.4,
    'zExp': 12.5, 'sExp': 8.289e-3, 'kExp': 0.4816, 'softRatio': 0.0025,
    'softLimit': 20, 'hornRatio': 0.0065, 'fluenceResampling': 3,
    'energy_weights': {"0.5": 0.08196, "1.0": 0.12385, "1.5": 0.10605, "2.0": 0.08307,
                       "2.5": 0.05881, "3.0": 0.03911, "3.5": 0.02131, "4.0": 0.02426,
                       "4.5": 0.0, "5.0": 0.00881, "5.5": 0.0, "6.0": 0.00498},
}


def main():
    from oracle import build_ref, oracle
    build_ref.compile_all()
    try:
        import tqdm  # noqa: F401
    except ImportError:
        sys.modules["tqdm"] = types.SimpleNamespace(tqdm=lambda it, **kw: it)
    from conehead.convolve_c import convolve_c

    from conehead_gb300 import Block, Source
    from conehead_gb300.kernel import poly_kernel_tables
    from conehead_gb300.phantoms import water_phantom
    ph = water_phantom(40, 0.5)
    src = Source()
    src.gantry = 0
    src.collimator = 0
    blk = Block()
    blk.set_square(10)
    T = oracle.prologue(src, blk, ph, SETTINGS, oracle.MODE_F64)["terma"]
    K, thetas, phis = poly_kernel_tables(SETTINGS["energy_weights"])
    kernel = types.SimpleNamespace(cumulative={"{:.2f}".format(float(p)): K[j] for j, p in enumerate(phis)})
    dose = np.zeros(T.shape, dtype=np.float64)
    dims = np.array([float(s) for s in ph.spacing], dtype=np.float64)
    t0 = time.perf_counter()
    convolve_c(np.ascontiguousarray(T), dose, dims, np.asarray(thetas, dtype=np.float64),
               np.asarray(phis, dtype=np.float64), kernel)
    dt = time.perf_counter() - t0
    cpu = None
    try:
        import subprocess
        for line in subprocess.run(["lscpu"], capture_output=True, text=True).stdout.splitlines():
            if line.startswith("Model name:"):
                cpu = line.split(":", 1)[1].strip()
    except OSError:
        pass
    print(json.dumps({"datum": "conehead convolve_c (Cython, as shipped)", "seconds": dt, "threads": 1,
                      "terma_voxels": int((T > 0).sum()), "grid": list(T.shape), "spacing_cm": 0.5,
                      "directions": [len(thetas), len(phis)], "dose_max": float(dose.max()),
                      "cpu": cpu, "machine": platform.machine()}))


if __name__ == "__main__":
    main()
