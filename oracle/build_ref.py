"""Compile conehead's own Cython DDA into oracle/_ref/ -- TEST INFRASTRUCTURE.

Recipe (no reference build system is used):
  1. Cython-translate the unmodified reference sources
       <ref>/conehead/vector.pyx  -> oracle/_ref/conehead/vector.c
       <ref>/conehead/dda_3d_c.pyx -> oracle/_ref/conehead/dda_3d_c.c
     with <ref> on the include path so their .pxd files resolve.
  2. Translate oracle/dda_ref_shim.pyx (a def wrapper around the nogil
     dda_3d_c) -> oracle/_ref/dda_ref_shim.c.
  3. gcc each .c into a CPython extension in oracle/_ref/.

Needs Cython (present in the build container, not on the GPU machine); the GPU
box never needs these modules -- they only generate the committed DDA golden
vectors in tests/golden/.  Usage:

    python oracle/build_ref.py [/path/to/conehead]
"""
import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")


def _cc(c_file, so_file):
    import numpy as np
    inc = [sysconfig.get_paths()["include"], np.get_include()]
    cmd = ["gcc", "-shared", "-fPIC", "-O2", "-w", "-o", so_file, c_file] + \
        [f"-I{p}" for p in inc]
    subprocess.run(cmd, check=True)


def build(ref_root="/root/reference"):
    src = os.path.join(ref_root, "conehead")
    pkg = os.path.join(OUT, "conehead")
    os.makedirs(pkg, exist_ok=True)
    open(os.path.join(pkg, "__init__.py"), "w").close()
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    for mod in ("vector", "dda_3d_c"):
        c_file = os.path.join(pkg, f"{mod}.c")
        subprocess.run([sys.executable, "-m", "cython", "-2", "-I", ref_root,
                        "--module-name", f"conehead.{mod}",
                        "-o", c_file, os.path.join(src, f"{mod}.pyx")], check=True)
        _cc(c_file, os.path.join(pkg, f"{mod}{ext}"))
    shim_c = os.path.join(OUT, "dda_ref_shim.c")
    subprocess.run([sys.executable, "-m", "cython", "-3", "-I", ref_root,
                    "-o", shim_c, os.path.join(HERE, "dda_ref_shim.pyx")], check=True)
    _cc(shim_c, os.path.join(OUT, f"dda_ref_shim{ext}"))
    return OUT


def load():
    """Import the compiled shim (after build())."""
    if OUT not in sys.path:
        sys.path.insert(0, OUT)
    import dda_ref_shim
    return dda_ref_shim


if __name__ == "__main__":
    build(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
    shim = load()
    print(shim.trace((1 / 14 ** .5, 2 / 14 ** .5, 3 / 14 ** .5), (101, 101, 101),
                     (50, 50, 50), (1.0, 1.0, 1.0))[1][:5])
