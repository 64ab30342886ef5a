"""In-tree build of libfvs2d_gb300.so for sm_103a.

Each translation unit is compiled by nvcc in parallel; the kernels are built
three times with different arithmetic flags (see csrc/fvs_kern_*.cu).  Host
code is compiled with -ffp-contract=off so that the setup arithmetic (edge
geometry, stencil coefficients) rounds exactly like the reference's source
order on both x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfvs2d_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE]
UNITS = {
    "fvs_setup.cpp": [],
    "fvs_capi.cu": [],
    "fvs_kern_strict.cu": ["-fmad=false"],
    "fvs_kern_fast.cu": ["-fmad=true"],
    "fvs_kern_mixed.cu": ["-fmad=true"],
    "fvs_kern_df.cu": ["-fmad=true"],
    "fvs_kern_bounds.cu": ["-fmad=true"],
    "fvs_noalloc.cu": [],
    "fvs_batch.cu": [],
    "fvs_mlp.cu": [],
}
HEADERS = ["fvs_internal.hpp", "fvs_kernels.cuh", "fvs_layout.hpp", "fvs_tiles.hpp", "df64.cuh", "fp64_fast.cuh",
           "fvs_tcgemm.cuh"]


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    for c in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fvs2d_gb300")


def _newest_dep() -> float:
    deps = [os.path.join(CSRC, f) for f in list(UNITS) + HEADERS]
    deps.append(os.path.join(INCLUDE, "fvs2d.h"))
    deps.append(os.path.abspath(__file__))
    return max(os.path.getmtime(d) for d in deps)


def _compile(src: str, extra: list) -> str:
    obj = os.path.join(BUILD, src + ".o")
    cmd = [nvcc(), *COMMON, *ARCH, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False) -> str:
    """Compile (if stale) and return the path of libfvs2d_gb300.so."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_dep():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(*kv), UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
