"""The C-ABI driven from a compiled C program (tests/c_host/fvs_c_host.c).

The Fortran host binds the same entry points through ISO_C_BINDING; no
Fortran compiler exists here, so a C99 program stands in for it.  On the CPU
the program must compile with every warning as an error against
include/fvs2d.h and link against the library.  On the GPU it runs the
drop-in for time_integration on a free-stream box with a perturbed state,
and its result is compared with the CPU oracle's steps of the same case:
bit-identical in strict FP64 (no transcendental function in the case).
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from fvs2d_gb300 import PREC_FP64, PREC_FP64_STRICT, Options, capi, meshgen
from fvs2d_gb300.sweep import Case, free_stream_state
from oracle_lib import Oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_host", "fvs_c_host.c")
MACH, AOA, DT = 0.5, 1.5, 0.02


def compile_host(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    libdir = os.path.dirname(capi.library_path())
    capi.load()  # builds the library if it is missing
    exe = str(tmp_path / "fvs_c_host")
    cmd = [cc, "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", libdir, "-lfvs2d_gb300", f"-Wl,-rpath,{libdir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def write_case(path, mesh, u0):
    a = capi.MeshArrays(mesh)
    nb = len(mesh.bndry_cells)
    hdr = np.array([a.node_xy.shape[0], a.tri.shape[0], a.quad.shape[0], nb, int(a.bn[:nb].sum())], np.int32)
    with open(path, "wb") as f:
        for arr in (hdr, a.node_xy, a.tri, a.quad, a.bn[:nb], a.bt[:nb], a.bc[: int(a.bn[:nb].sum())],
                    np.array([MACH, AOA, DT]), np.ascontiguousarray(u0, np.float64)):
            f.write(np.ascontiguousarray(arr).tobytes())


def case():
    mesh = meshgen.dirichlet_square(12, 12, jitter=0.15, bc="freestream")
    u0 = free_stream_state(Case(0, 0, MACH, AOA), mesh.ncells)
    x = np.linspace(0.0, 1.0, mesh.ncells)
    u0[:, 0] *= 1.0 + 0.05 * np.sin(7.0 * x)
    u0[:, 3] *= 1.0 + 0.03 * np.cos(5.0 * x)
    return mesh, u0


def test_c_host_compiles_and_links(tmp_path):
    exe = compile_host(tmp_path)
    r = subprocess.run([exe, str(tmp_path / "missing.bin"), str(tmp_path / "out.bin"), "3", "0"],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "cannot read" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [PREC_FP64_STRICT, PREC_FP64])
def test_c_host_matches_oracle(tmp_path, prec):
    exe = compile_host(tmp_path)
    mesh, u0 = case()
    write_case(tmp_path / "case.bin", mesh, u0)
    nsteps = 5
    r = subprocess.run([exe, str(tmp_path / "case.bin"), str(tmp_path / "out.bin"), str(nsteps), str(prec)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(tmp_path / "out.bin", np.float64).reshape(mesh.ncells, 4)
    norms = np.array([[float(v) for v in line.split()] for line in r.stdout.strip().splitlines()])
    o = Oracle(mesh, Options(mach_inf=MACH, aoa_inf_deg=AOA, dt=DT, steady=False))
    o.cvar = u0
    ref_norms = o.time_integration(0.0, nsteps)
    ref = o.cvar
    o.close()
    if prec == PREC_FP64_STRICT:
        assert np.array_equal(got, ref), float(np.abs(got - ref).max())
        assert np.allclose(norms, ref_norms, rtol=1e-13, atol=0)
    else:
        assert float(np.abs(got - ref).max() / np.abs(ref).max()) <= 1e-12
        assert np.allclose(norms, ref_norms, rtol=1e-9, atol=0)
