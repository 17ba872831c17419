"""Build libesmcuda.so for sm_103a with nvcc (no cmake): the translation units compiled in
parallel -- the C ABI, the FP32 kernels (the production build, with the approximate single-precision
division: 2 ulp, 12 % faster line moves at the benchmarked size), the FP64 kernels (the parity build
without FMA contraction and with IEEE division, like the CPU oracle) and the surrogate MLP -- then
linked into one shared library, in-tree.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libesmcuda.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
BASE = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]
UNITS = [("esm_capi.cu", []), ("esm_f32.cu", ["-prec-div=false"]), ("esm_f64.cu", ["-fmad=false"]), ("esm_mlp.cu", [])]


def nvcc():
    for p in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if p and (os.path.sep not in p or os.path.exists(p)):
            return p
    return "nvcc"


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(os.path.dirname(PKG), "include", "esmcuda.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False):
    """Compile and link; returns the library path. Raises on a compiler error."""
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()

    def one(unit):
        src, extra = unit
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *BASE, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(one, UNITS))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
