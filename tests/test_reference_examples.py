"""The reference's two shipped example cases through the device path.

examples/isentropic_vortex (7,226 triangles, Dirichlet exact-vortex boundary,
src/residual.f90:210-216; LSQ-fn; classic 4-stage RK of order 4, dt 0.01) and
examples/naca0012_ogrid (65,536 quadrilaterals, slip wall + free stream;
LSQ-nn; SSP-RK(4,2) steady with local time steps at CFL 1.25,
src/runge_kutta.f90:349-418) are read from the committed fixture
tests/golden/reference_examples.npz (written by make_reference_examples.py
from the reference's .grid, .bc, fvs2d.input and fvs2d.vortex files), with
the scheme exactly as the reference's input parser sets it.

CPU: the fixture equals what the parsers read from the reference's files
(where the reference is mounted), and the oracle reproduces the fixture's
digests of its 20-step run on the machine type that wrote them.

GPU: 20 steps from initialize_solution, then compute_residual at the final
time, against the oracle run live on the same host.  The conserved state
and ws_nrml are compared relative to max|ref|.  The residual is compared
relative to the magnitude of the face fluxes it sums, S = max over cells of
ws_nrml / vol * max|U|: in these examples the residual is a near-
cancellation of those fluxes (max|resid| is 7e-4 S for the weak, slow
vortex and 2.7e-3 S twenty steps from the free stream around the airfoil),
so relative to max|resid| the same differences read 400-1400x larger
(measured: 3e-13 strict vortex, 7e-12 double-float vortex, 1.5e-4 mixed
vortex).
  FP64_STRICT  bit-identical; for the vortex, whose Dirichlet ghost states
               call exp and pow (CUDA's against glibc's), state and ws_nrml
               1e-13 of max|ref| and residual 1e-13 S; norms rtol 1e-13
  FP64         state and ws_nrml 1e-12 of max|ref| after all 20 steps (the
               bar is 1e-12 per step), residual 1e-12 S; norms rtol 1e-9
  FP64_DF      the same bars as FP64
  MIXED        state 1e-5 of max|ref|, ws_nrml 1e-5, residual 1e-5 S;
               norms rtol 1e-3
"""
import os
import platform
import sys

import numpy as np
import pytest

from fvs2d_gb300 import PREC_FP64, PREC_FP64_DF, PREC_FP64_STRICT, PREC_MIXED, Solver

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_reference_examples as M  # noqa: E402

NAMES = sorted(M.EXAMPLES)
# digests of the oracle's run were written on this machine type
FIXTURE_MACHINE = "x86_64"


def fixture():
    return np.load(M.OUT)


def case(name):
    with fixture() as z:
        return M.unpack(z, name)


@pytest.mark.parametrize("name", NAMES)
def test_fixture_is_the_reference_example(name, reference_examples):
    ref_root = os.path.dirname(reference_examples)
    mesh, opt = M.read_example(ref_root, name)
    got_mesh, got_opt = case(name)
    assert np.array_equal(got_mesh.node_xy, mesh.node_xy)
    assert np.array_equal(got_mesh.tri_nodes, mesh.tri_nodes.reshape(-1, 3))
    assert np.array_equal(got_mesh.quad_nodes, mesh.quad_nodes.reshape(-1, 4))
    assert got_mesh.bndry_types == list(mesh.bndry_types)
    assert all(np.array_equal(a, b) for a, b in zip(got_mesh.bndry_cells, mesh.bndry_cells))
    assert got_opt == opt


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_example_digests(name):
    if platform.machine() != FIXTURE_MACHINE:
        pytest.skip(f"digests written on {FIXTURE_MACHINE} (libm's exp/pow round differently elsewhere)")
    mesh, opt = case(name)
    r = M.oracle_run(mesh, opt, nthreads=os.cpu_count() or 1)
    with fixture() as z:
        assert np.array_equal(r["norms"], z[name + "/norms"])
        assert M.digest(r["state"]) == str(z[name + "/digest_state"])
        assert M.digest(r["resid"], r["ws"]) == str(z[name + "/digest_residual"])


_ORACLE = {}


def oracle(name):
    if name not in _ORACLE:
        mesh, opt = case(name)
        _ORACLE[name] = M.oracle_run(mesh, opt, nthreads=os.cpu_count() or 1)
    return _ORACLE[name]


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [PREC_FP64_STRICT, PREC_FP64, PREC_FP64_DF, PREC_MIXED])
@pytest.mark.parametrize("name", NAMES)
def test_gpu_runs_reference_example(name, prec):
    mesh, opt = case(name)
    want = oracle(name)
    with Solver(mesh, opt.replace(precision=prec)) as s:
        s.initialize_solution()
        # the library's host initial state against the oracle's, then the
        # oracle's exact start so that the runs begin from the same bits
        assert rel(s.cvar, want["start"]) <= 1e-15
        s.cvar = want["start"]
        norms = s.time_integration(0.0, M.STEPS)
        state = s.cvar
        resid, ws = s.compute_residual(want["t_end"])
    errs = {"state": rel(state, want["state"]), "ws": rel(ws, want["ws"]),
            "resid": float(np.abs(resid - want["resid"]).max() / want["flux_scale"]),
            "resid_vs_max": rel(resid, want["resid"])}
    if prec == PREC_FP64_STRICT:
        if opt.vortex:
            assert max(errs["state"], errs["ws"], errs["resid"]) <= 1e-13, errs
        else:
            assert np.array_equal(state, want["state"]), errs
            assert np.array_equal(resid, want["resid"]), errs
            assert np.array_equal(ws, want["ws"]), errs
        assert np.allclose(norms, want["norms"], rtol=1e-13, atol=0)
    elif prec in (PREC_FP64, PREC_FP64_DF):
        assert max(errs["state"], errs["ws"], errs["resid"]) <= 1e-12, errs
        assert np.allclose(norms, want["norms"], rtol=1e-9, atol=0)
    else:
        assert max(errs["state"], errs["ws"], errs["resid"]) <= 1e-5, errs
        assert np.allclose(norms, want["norms"], rtol=1e-3, atol=0)
