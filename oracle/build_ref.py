"""Build the reference's own ILU(0) kernel from its source -- TEST INFRASTRUCTURE ONLY.

The reference's compiled piece on this path is ``aquaflux/solve/_ilu0.pyx`` (Cython; its build is
``setup.py:32-38``: ``cythonize`` with ``language_level="3"`` and numpy's include directory).  This
recipe builds that file, untouched, into ``oracle/_ref/`` (git-ignored: generated and compiled
code never enters the repository), in two steps that can run on different machines:

1. where the reference checkout and Cython are present: ``cython -3`` the ``.pyx`` into
   ``oracle/_ref/_ilu0.c``;
2. where ``oracle/_ref/_ilu0.c`` is present: compile it against this interpreter's headers and
   numpy's into ``oracle/_ref/_ilu0<EXT_SUFFIX>``.

Compiled with ``-ffp-contract=off``: the kernel's loops then round as written (no fused
multiply-add), the arithmetic of its pure-Python twin (``aquaflux/solve/ilu0.py:76-150``) and of
the GPU factor it pins.  The module is the checker of the GPU ILU(0) (bitwise factor and transposed
solve) and the timed CPU baseline of ``bench.py``'s ILU(0) comparison; nothing in the package
imports it.

Usage: ``python oracle/build_ref.py [reference checkout]`` (default ``AQUAFLUX_REFERENCE``, else
``/root/reference``).
"""
from __future__ import annotations

import importlib.util
import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
C_FILE = os.path.join(OUT, "_ilu0.c")
SO_FILE = os.path.join(OUT, "_ilu0" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))


def _reference_root(arg: str | None) -> str:
    return arg or os.environ.get("AQUAFLUX_REFERENCE") or "/root/reference"


def generate_c(reference: str | None = None) -> bool:
    """Step 1: cythonize the reference's ``_ilu0.pyx`` (True when ``_ilu0.c`` is up to date)."""
    pyx = os.path.join(_reference_root(reference), "aquaflux", "solve", "_ilu0.pyx")
    if not os.path.exists(pyx):
        return os.path.exists(C_FILE)
    if os.path.exists(C_FILE) and os.path.getmtime(C_FILE) >= os.path.getmtime(pyx):
        return True
    try:
        import Cython  # noqa: F401
    except ImportError:
        return os.path.exists(C_FILE)
    os.makedirs(OUT, exist_ok=True)
    r = subprocess.run([sys.executable, "-m", "cython", "-3", pyx, "-o", C_FILE],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"cython failed on {pyx}:\n{r.stderr[-2000:]}")
    return True


def compile_so() -> str | None:
    """Step 2: compile ``_ilu0.c`` into an extension module; its path, or None without the C."""
    if not os.path.exists(C_FILE):
        return None
    if os.path.exists(SO_FILE) and os.path.getmtime(SO_FILE) >= os.path.getmtime(C_FILE):
        return SO_FILE
    import numpy as np

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        return None
    cmd = [cc, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fno-strict-aliasing", "-fwrapv",
           "-I", sysconfig.get_paths()["include"], "-I", np.get_include(), C_FILE, "-o", SO_FILE]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling {C_FILE} failed:\n{r.stderr[-2000:]}")
    return SO_FILE


def build_ref(reference: str | None = None) -> str | None:
    """Both steps as far as this machine allows; the module path or None."""
    generate_c(reference)
    return compile_so()


def load_ref():
    """The compiled reference module (``diagonal_positions``, ``factor``, ``solve``,
    ``solve_transpose``), or None when it is not built here."""
    if not os.path.exists(SO_FILE):
        return None
    spec = importlib.util.spec_from_file_location("_ilu0", SO_FILE)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


if __name__ == "__main__":
    print(build_ref(sys.argv[1] if len(sys.argv) > 1 else None))
