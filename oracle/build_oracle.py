"""Build recipe of the CPU oracle (test infrastructure only).

gcc -O2 -ffp-contract=off: no multiply-add fusion, so the oracle rounds every
product and sum exactly as the Fortran source writes it, on x86-64 and on
aarch64 alike.  OpenMP drives the race-free multi-threaded residual used as
the timed CPU baseline.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "build")
LIB = os.path.join(OUT_DIR, "libfvs_oracle.so")
SRC = [os.path.join(HERE, "fvs_oracle.c")]
DEPS = SRC + [os.path.join(HERE, "fvs_oracle.h"), os.path.join(os.path.dirname(HERE), "include", "fvs2d.h"),
              os.path.abspath(__file__)]
CFLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function"]


def build(force: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in DEPS):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["gcc", *CFLAGS, "-shared", "-o", tmp, *SRC, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
