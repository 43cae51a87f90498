"""Build libgbhydro.so for sm_103a with nvcc (no cmake).

Translation units are compiled in parallel; the FP64 units use -fmad=false
so that no fused multiply-add changes their rounding relative to the CPU
oracle. Outputs land in torch_gb300/_build/ and torch_gb300/libgbhydro.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbhydro.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# unit -> extra flags (the mixed unit's FP32 reconstruction and Riemann
# arithmetic uses the approximate FP32 division and square root: a few ulp
# against the correctly rounded ones, far inside the mixed path's
# tolerance; its FP64 update is unaffected)
UNITS = {
    "capi.cu": ["-fmad=false"],
    "cool.cu": ["-fmad=false"],
    "hydro_fp64.cu": ["-fmad=false"],
    "hydro_mixed.cu": ["-prec-div=false", "-prec-sqrt=false"],
    "mlp.cu": [],
    "noalloc.cu": ["-fmad=false"],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps_mtime() -> float:
    m = 0.0
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    base = [nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
            "-I", os.path.join(ROOT, "include"), "-I", CSRC, "--expt-relaxed-constexpr",
            "-Xptxas", "-warn-spills" if verbose else "-O3"]

    def one(u):
        obj = os.path.join(BUILD, u.replace(".cu", ".o"))
        cmd = base + UNITS[u] + ["-c", os.path.join(CSRC, u), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(one, units))
    tmp = LIB + ".tmp"
    r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
