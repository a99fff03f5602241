"""Builds the CUDA library in-tree: fall3d_gb300/libfall3d_gb300.so.

One nvcc invocation per translation unit, in parallel, for sm_103a only
(-gencode arch=compute_103a,code=sm_103a).  The binary64 translation units
are compiled with --fmad=false so that no multiply-add is contracted: the
plain form must round every operation as the reference's Fortran does.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfall3d_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]
# translation unit -> extra flags
UNITS = {
    "f3d_transport.cu": ["--fmad=false"],
    "f3d_budget.cu": ["--fmad=false"],
    "f3d_coeff.cu": ["--fmad=false"],
    "f3d_fused.cu": ["--fmad=false"],
    "f3d_fused2.cu": ["--fmad=false"],
    "f3d_api.cu": ["--fmad=false", "-Xcompiler", "-fvisibility=default"],
    "f3d_ctx.cu": ["--fmad=false", "-Xcompiler", "-fvisibility=default"],
    "f3d_batch.cu": ["--fmad=false", "-Xcompiler", "-fvisibility=default"],
    "f3d_serve.cu": ["-Xcompiler", "-fvisibility=default"],
    "f3d_output.cu": ["--fmad=false", "-Xcompiler", "-fvisibility=default"],
    "f3d_gravity.cu": ["--fmad=false", "-Xcompiler", "-fvisibility=default"],
    "f3d_aggregation.cu": ["--fmad=false", "-Xcompiler", "-fvisibility=default"],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps(unit: str):
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + [
        os.path.join(INCLUDE, "fall3d_gpu.h"), os.path.join(CSRC, unit), __file__]


def _compile(unit: str, flags, verbose=False) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in _deps(unit)):
        return obj
    cmd = [nvcc(), *ARCH, *COMMON, *flags, "-c", src, "-o", obj + ".tmp"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr}\n{r.stdout}")
    if verbose:
        sys.stderr.write(r.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    tmp = LIB + f".{os.getpid()}.tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}\n{r.stdout}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
