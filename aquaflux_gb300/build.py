"""In-tree build of ``libfvgb.so`` for sm_103a (and of the CPU oracle's C restatement).

``nvcc`` compiles the translation units in parallel (one ``-gencode``), then links a shared
library with a static CUDA runtime, so it loads beside any torch build.  ``sparse.cu`` is compiled
with ``-fmad=false``: its fp64 ILU(0) must round exactly like the reference's sequential kernel;
``noalloc.cu`` too, so that its transposed SpMV rounds like ``sparse.cu``'s (bitwise the same).
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
UNITS = {"mesh.cu": [], "residual.cu": [], "capi.cu": [], "sparse.cu": ["-fmad=false"],
         "colour.cu": [], "noalloc.cu": ["-fmad=false"], "amg.cu": [], "krylov.cu": [], "rcm.cu": []}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def build_library(verbose: bool = False) -> str:
    nvcc = _nvcc()
    obj_dir = os.path.join(HERE, "_build")
    os.makedirs(obj_dir, exist_ok=True)
    out = os.path.join(HERE, "libfvgb.so")
    srcs = [os.path.join(CSRC, u) for u in UNITS]
    deps = srcs + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".cuh")] + \
        [os.path.join(ROOT, "include", "fvgb.h")]
    if os.path.exists(out) and os.path.getmtime(out) > max(os.path.getmtime(d) for d in deps):
        return out

    def compile_one(unit):
        src = os.path.join(CSRC, unit)
        obj = os.path.join(obj_dir, unit.replace(".cu", ".o"))
        cmd = [nvcc, ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
               "-I", os.path.join(ROOT, "include"), *UNITS[unit], "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {unit}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = out + ".tmp"
    cmd = [nvcc, ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, out)
    return out


def build_oracle() -> None:
    """Compile the test checkers: the oracle's C restatement of the ILU(0) kernel, and the
    reference's own ILU(0) kernel from its source where this machine has it (``oracle/_ref``;
    a failure there only leaves the checker unbuilt)."""
    import sys

    script = os.path.join(ROOT, "oracle", "build_oracle.py")
    if os.path.exists(script):
        subprocess.run([sys.executable, script], check=True, stdout=subprocess.DEVNULL)
    ref = os.path.join(ROOT, "oracle", "build_ref.py")
    if os.path.exists(ref):
        subprocess.run([sys.executable, ref], check=False, stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL)
