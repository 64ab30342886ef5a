"""Build recipe of the CPU oracle (test infrastructure only).

The checker: gcc -O2 -ffp-contract=off, no multiply-add fusion, so the oracle
rounds every product and sum exactly as the Fortran source writes it, on
x86-64 and on aarch64 alike.

The timed CPU baseline: the same source with -O3 -ffast-math, as the
reference itself is compiled with -Ofast (CMakeLists.txt:32), so that the
baseline is timed at the optimisation level the reference ships with.  Its
results are not bit-exact and it checks nothing.  OpenMP drives the
race-free multi-threaded residual in both.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "build")
LIB = os.path.join(OUT_DIR, "libfvs_oracle.so")
LIB_TIMED = os.path.join(OUT_DIR, "libfvs_oracle_timed.so")
SRC = [os.path.join(HERE, "fvs_oracle.c")]
DEPS = SRC + [os.path.join(HERE, "fvs_oracle.h"), os.path.join(os.path.dirname(HERE), "include", "fvs2d.h"),
              os.path.abspath(__file__)]
CFLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function"]
CFLAGS_TIMED = ["-O3", "-std=c11", "-ffast-math", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function"]


def build(force: bool = False, timed: bool = False) -> str:
    """The checker's library, or (timed) the baseline's."""
    lib, flags = (LIB_TIMED, CFLAGS_TIMED) if timed else (LIB, CFLAGS)
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= max(os.path.getmtime(d) for d in DEPS):
        return lib
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = lib + ".tmp"
    cmd = ["gcc", *flags, "-shared", "-o", tmp, *SRC, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force=True))
    print(build(force=True, timed=True))
