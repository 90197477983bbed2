"""Build the CPU checkers -- TEST INFRASTRUCTURE ONLY.

1. ``oracle/libilu0_oracle.so`` from ``oracle/ilu0_oracle.c`` (the plain-C restatement of the
   reference's ILU(0) kernel), with ``-ffp-contract=off`` so no multiply-add is fused.
2. ``oracle/_ref/_ilu0*.so``: the reference's OWN compiled kernel, built from its source
   ``aquaflux/solve/_ilu0.pyx`` where it lies.  When the reference tree and Cython are available
   (the development container) the ``.pyx`` is translated to ``oracle/_ref/_ilu0.c``; that C file
   (not the reference source) travels with the working tree, so a machine without the reference or
   Cython (the GPU machine) still compiles the same kernel from it.  Nothing here is committed:
   ``oracle/_ref/`` and ``*.so`` are git-ignored.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
REF_PYX = "/root/reference/aquaflux/solve/_ilu0.pyx"
REF_DIR = os.path.join(HERE, "_ref")


def build_c_oracle() -> str:
    out = os.path.join(HERE, "libilu0_oracle.so")
    src = os.path.join(HERE, "ilu0_oracle.c")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", out],
                       check=True)
    return out


def build_reference_kernel() -> str | None:
    os.makedirs(REF_DIR, exist_ok=True)
    c_file = os.path.join(REF_DIR, "_ilu0.c")
    if os.path.exists(REF_PYX):
        try:
            import Cython  # noqa: F401
        except ImportError:
            Cython = None
        if Cython is not None and (not os.path.exists(c_file)
                                   or os.path.getmtime(c_file) < os.path.getmtime(REF_PYX)):
            shutil.copy(REF_PYX, os.path.join(REF_DIR, "_ilu0.pyx"))
            subprocess.run([sys.executable, "-m", "cython", "-3", "-o", c_file,
                            os.path.join(REF_DIR, "_ilu0.pyx")], check=True,
                           capture_output=True)
            os.remove(os.path.join(REF_DIR, "_ilu0.pyx"))
    if not os.path.exists(c_file):
        return None
    import numpy

    ext = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    out = os.path.join(REF_DIR, "_ilu0" + ext)
    if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(c_file):
        return out
    inc = [sysconfig.get_paths()["include"], numpy.get_include()]
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fno-strict-aliasing",
           *[f"-I{i}" for i in inc], c_file, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        print("reference ILU(0) kernel did not build:", r.stderr[-2000:])
        return None
    return out


if __name__ == "__main__":
    print(build_c_oracle())
    print(build_reference_kernel())
