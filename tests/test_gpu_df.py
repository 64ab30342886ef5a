"""Double-float path (FVS_PREC_FP64_DF) vs the CPU oracle.

Gradient, limiter, reconstruction, Roe flux, the residual gather and the RK
stage run in pairs of FP32 numbers (48-bit significand, relative precision
2^-48 per operation against FP64's 2^-53); the state is stored in FP64 and
the norms are summed as FP32 pairs.
The bar is the FP64 drop-in's: max|diff| <= 1e-12 * max|ref| per residual,
gradient and step; the limiter value itself is held to 1e-11.
"""
import numpy as np
import pytest

import cases
from fvs2d_gb300 import PREC_FP64_DF, Solver
from fvs2d_gb300.batch import Batch
from oracle_lib import Oracle
from test_gpu_parity import INTEGRATOR_CASES, STRICT_RESIDUAL_CASES, _perturbed_state, rel

pytestmark = pytest.mark.gpu

TOL = 1e-12


# The reference's "Van Albada" variant returns unbounded limiter values
# (src/gradient_limiter.f90:122-127): on the airfoil case ~3 % of the face
# states leave the physical range and which residuals become non-finite
# depends on the last bits.  The strict test covers it bit-exactly.
DF_RESIDUAL_CASES = sorted(k for k in STRICT_RESIDUAL_CASES if k != "airfoil_albada")


@pytest.mark.parametrize("name", DF_RESIDUAL_CASES)
def test_residual_df(name):
    mesh, opt = STRICT_RESIDUAL_CASES[name]()
    orc = Oracle(mesh, opt)
    u = _perturbed_state(orc)
    orc.cvar = u
    r_ref, w_ref = orc.compute_residual(0.0)
    g_ref, phi_ref = orc.gradient()
    with Solver(mesh, opt.replace(precision=PREC_FP64_DF)) as s:
        s.cvar = u
        r, w = s.compute_residual(0.0)
        g, phi = s.gradient()
    assert np.isfinite(r).all() and np.isfinite(r_ref).all()
    assert rel(g, g_ref) <= TOL, rel(g, g_ref)
    assert rel(r, r_ref) <= TOL, rel(r, r_ref)
    assert rel(w, w_ref) <= TOL, rel(w, w_ref)
    # the limiter divides face differences that nearly cancel, which
    # amplifies the 2^-48 operation error: 1e-11 on phi itself
    assert rel(phi, phi_ref) <= 1e-11, rel(phi, phi_ref)


@pytest.mark.parametrize("name", ["dirichlet_vortex", "mms"])
def test_residual_dirichlet_df(name):
    mesh, opt = cases.dirichlet_vortex() if name == "dirichlet_vortex" else cases.mms_box()
    orc = Oracle(mesh, opt)
    orc.initialize_solution()
    r_ref, w_ref = orc.compute_residual(0.37)
    with Solver(mesh, opt.replace(precision=PREC_FP64_DF)) as s:
        s.initialize_solution()
        r, w = s.compute_residual(0.37)
    assert rel(r, r_ref) <= TOL and rel(w, w_ref) <= TOL, (rel(r, r_ref), rel(w, w_ref))


@pytest.mark.parametrize("name", sorted(INTEGRATOR_CASES))
def test_time_integration_df(name):
    factory, nsteps, _ = INTEGRATOR_CASES[name]
    mesh, opt = factory()
    orc = Oracle(mesh, opt)
    orc.initialize_solution()
    u0 = orc.cvar
    n_ref = orc.time_integration(0.0, nsteps)
    u_ref = orc.cvar
    with Solver(mesh, opt.replace(precision=PREC_FP64_DF)) as s:
        s.cvar = u0
        n = s.time_integration(0.0, nsteps)
        u = s.cvar
    assert rel(u, u_ref) <= TOL, rel(u, u_ref)
    assert np.allclose(n, n_ref, rtol=1e-8), (n, n_ref)


def test_full_size_df_conservation_and_oracle():
    """1,048,576 cells: one DF step against the oracle, conservation, and
    determinism of two runs."""
    from fvs2d_gb300 import meshgen
    mesh = meshgen.periodic_square(1024, 512, jitter=0.2, seed=1, jitter_seed=2)
    _, opt = cases.periodic_vortex(4)
    orc = Oracle(mesh, opt, nthreads=8)
    orc.initialize_solution()
    u0 = orc.cvar
    orc.time_integration(0.0, 1)
    u_ref = orc.cvar
    with Solver(mesh, opt.replace(precision=PREC_FP64_DF)) as s:
        s.cvar = u0
        vol = s.export("cell_vol")
        s.time_integration(0.0, 1)
        u1 = s.cvar
        s.cvar = u0
        s.time_integration(0.0, 1)
        u2 = s.cvar
    assert np.array_equal(u1, u2)
    assert rel(u1, u_ref) <= TOL, rel(u1, u_ref)
    tot0 = (vol[:, None] * u0).sum(0)
    tot1 = (vol[:, None] * u1).sum(0)
    assert np.all(np.abs(tot1 - tot0) <= 1e-11 * np.abs(tot0).max()), (tot0, tot1)


def test_batch_df_matches_single():
    specs = [(48, 16, 0.5, 0.0), (64, 20, 0.75, 1.5)]
    meshes, opts = [], []
    for nw, nr, mach, aoa in specs:
        m, o = cases.airfoil(nw=nw, nr=nr, cfl=0.5, mach_inf=mach, aoa_inf_deg=aoa, precision=PREC_FP64_DF)
        meshes.append(m)
        opts.append(o)
    with Batch(meshes, opts) as b:
        b.initialize_solution()
        b.steps(5)
        got = [b.get_state(c) for c in range(2)]
    for c in range(2):
        with Solver(meshes[c], opts[c]) as s:
            s.initialize_solution()
            s.time_integration(0.0, 5)
            assert rel(got[c], s.cvar) <= 1e-13, rel(got[c], s.cvar)
