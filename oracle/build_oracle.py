"""Build the CPU checker -- TEST INFRASTRUCTURE ONLY.

``oracle/libilu0_oracle.so`` from ``oracle/ilu0_oracle.c`` (the plain-C restatement of the
reference's ILU(0) kernel), with ``-ffp-contract=off`` so no multiply-add is fused.  The
reference's own kernel is Cython (``aquaflux/solve/_ilu0.pyx``): compiling it needs generated C,
so it is not built here; the restatement is pinned to the reference's pure-Python twin
(``aquaflux/solve/ilu0.py:76-150``) through the committed fixture ``tests/golden/ilu0.npz``.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def build_c_oracle() -> str:
    out = os.path.join(HERE, "libilu0_oracle.so")
    src = os.path.join(HERE, "ilu0_oracle.c")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", out],
                       check=True)
    return out


if __name__ == "__main__":
    print(build_c_oracle())
