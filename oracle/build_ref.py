"""Compile conehead's own Cython DDA and cone convolution into oracle/_ref/
-- TEST INFRASTRUCTURE.

Recipe (no reference build system is used):
  1. translate(): Cython-translate the unmodified reference sources
       <ref>/conehead/vector.pyx     -> oracle/_ref/conehead/vector.c
       <ref>/conehead/dda_3d_c.pyx   -> oracle/_ref/conehead/dda_3d_c.c
       <ref>/conehead/convolve_c.pyx -> oracle/_ref/conehead/convolve_c.c
     with <ref> on the include path so their .pxd files resolve, and
     oracle/dda_ref_shim.pyx (a def wrapper around the nogil dda_3d_c) ->
     oracle/_ref/dda_ref_shim.c.  Needs Cython and the reference sources.
  2. compile_all(): gcc each translated .c into a CPython extension in
     oracle/_ref/ for this interpreter (the file name carries the platform, so
     x86_64 and aarch64 builds sit side by side).  Needs only gcc, the Python
     headers and numpy: it also runs where the translated .c files were
     copied without the reference sources or Cython (the GPU host).

The DDA modules generate the committed DDA golden vectors in tests/golden/;
convolve_c is timed as a datum by oracle/time_convolve_c.py.  Usage:

    python oracle/build_ref.py /path/to/conehead
    CONEHEAD_REFERENCE=/path/to/conehead python oracle/build_ref.py
    python oracle/build_ref.py --compile-only
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


def reference_root(arg=None):
    """The conehead checkout: the argument, else $CONEHEAD_REFERENCE."""
    root = arg or os.environ.get("CONEHEAD_REFERENCE")
    if not root:
        raise SystemExit("name the conehead checkout as an argument or in CONEHEAD_REFERENCE")
    return root


MODULES = ("vector", "dda_3d_c", "convolve_c")


def translate(ref_root):
    src = os.path.join(ref_root, "conehead")
    pkg = os.path.join(OUT, "conehead")
    os.makedirs(pkg, exist_ok=True)
    for mod in MODULES:
        subprocess.run([sys.executable, "-m", "cython", "-2", "-I", ref_root,
                        "--module-name", f"conehead.{mod}",
                        "-o", os.path.join(pkg, f"{mod}.c"), os.path.join(src, f"{mod}.pyx")], check=True)
    subprocess.run([sys.executable, "-m", "cython", "-3", "-I", ref_root,
                    "-o", os.path.join(OUT, "dda_ref_shim.c"), os.path.join(HERE, "dda_ref_shim.pyx")],
                   check=True)


def compile_all():
    """gcc every translated module that is missing or older than its .c."""
    pkg = os.path.join(OUT, "conehead")
    os.makedirs(pkg, exist_ok=True)
    open(os.path.join(pkg, "__init__.py"), "a").close()
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    jobs = [(os.path.join(pkg, f"{m}.c"), os.path.join(pkg, f"{m}{ext}")) for m in MODULES]
    jobs.append((os.path.join(OUT, "dda_ref_shim.c"), os.path.join(OUT, f"dda_ref_shim{ext}")))
    for c_file, so_file in jobs:
        if not os.path.exists(c_file):
            raise FileNotFoundError(f"{c_file} is missing: run translate() where Cython and the sources are")
        if not os.path.exists(so_file) or os.path.getmtime(so_file) < os.path.getmtime(c_file):
            _cc(c_file, so_file)
    return OUT


def build(ref_root):
    translate(ref_root)
    return compile_all()


def load():
    """Import the compiled shim (after build())."""
    if OUT not in sys.path:
        sys.path.insert(0, OUT)
    import dda_ref_shim
    return dda_ref_shim


if __name__ == "__main__":
    if "--compile-only" in sys.argv:
        compile_all()
    else:
        build(reference_root(sys.argv[1] if len(sys.argv) > 1 else None))
    shim = load()
    print(shim.trace((1 / 14 ** .5, 2 / 14 ** .5, 3 / 14 ** .5), (101, 101, 101),
                     (50, 50, 50), (1.0, 1.0, 1.0))[1][:5])
