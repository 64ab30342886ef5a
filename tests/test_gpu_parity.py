"""Device path vs CPU oracle, through the C-ABI (fvs2d_gb300.Solver).

Tolerances, per arithmetic mode of the device path:
  FP64_STRICT  bit-identical (==) wherever no transcendental function runs;
               the exact-vortex / MMS Dirichlet ghost states call exp, pow and
               sin, whose CUDA and glibc implementations may differ in the last
               unit: max|diff| <= 1e-13 * max|ref| there.
  FP64         (FMA contraction) max|diff| <= 1e-12 * max|ref| per step.
  MIXED        (FP32 flux/gradient) state max|diff| <= 1e-6 * max|ref|.
Residual norms come from a blocked reduction (different summation order than
the oracle's sequential sum): relative 1e-13.
"""
import numpy as np
import pytest

import cases
from fvs2d_gb300 import PREC_FP64, PREC_FP64_STRICT, PREC_MIXED, FvsError, Solver, capi
from oracle_lib import Oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


STRICT_RESIDUAL_CASES = {
    "periodic_lsq_fn": lambda: cases.periodic_vortex(20, jitter=0.2),
    "periodic_lsq_nn_p1": lambda: cases.periodic_vortex(20, jitter=0.2, lsq_stencil="nn", lsq_pow=1.0),
    "periodic_ggcb": lambda: cases.periodic_vortex(20, jitter=0.2, grad_method=1),
    "periodic_ggnb": lambda: cases.periodic_vortex(20, jitter=0.2, grad_method=2),
    "periodic_umuscl": lambda: cases.periodic_vortex(20, jitter=0.2, reconst=3, umuscl=1.0 / 3.0),
    "periodic_first_order": lambda: cases.periodic_vortex(20, reconst=1),
    "airfoil_venk": lambda: cases.airfoil(),
    "airfoil_barth": lambda: cases.airfoil(limiter=2),
    "airfoil_albada": lambda: cases.airfoil(limiter=3),
    "airfoil_nn_nolim": lambda: cases.airfoil(lsq_stencil="nn", limiter=0),
    "mixed_tri_quad_lsq_fn": lambda: cases.periodic_mixed(),
    "mixed_tri_quad_ggcb": lambda: cases.periodic_mixed(grad_method=1),
    "mixed_tri_quad_ggnb": lambda: cases.periodic_mixed(grad_method=2),
    "quad_airfoil_venk": lambda: cases.airfoil_quads(),
    "quad_airfoil_nn": lambda: cases.airfoil_quads(lsq_stencil="nn", limiter=0),
}


def _perturbed_state(orc, seed=7):
    """Initial state plus a smooth seeded perturbation (exercises the limiter)."""
    orc.initialize_solution()
    u = orc.cvar
    rng = np.random.default_rng(seed)
    u = u * (1.0 + 0.02 * rng.standard_normal(u.shape))
    return u


@pytest.mark.parametrize("name", sorted(STRICT_RESIDUAL_CASES))
def test_residual_strict_bit_exact(name):
    mesh, opt = STRICT_RESIDUAL_CASES[name]()
    orc = Oracle(mesh, opt)
    u = _perturbed_state(orc)
    orc.cvar = u
    r_ref, w_ref = orc.compute_residual(0.0)
    g_ref, phi_ref = orc.gradient()
    with Solver(mesh, opt.replace(precision=PREC_FP64_STRICT)) as s:
        s.cvar = u
        r, w = s.compute_residual(0.0)
        g, phi = s.gradient()
    # NaN where the oracle has NaN: the reference's "Van Albada" variant can
    # return an unbounded limiter value (src/gradient_limiter.f90:122-127)
    assert np.array_equal(g, g_ref, equal_nan=True), f"gradient differs: {rel(g, g_ref):.3e}"
    assert np.array_equal(phi, phi_ref, equal_nan=True), f"limiter differs: {rel(phi, phi_ref):.3e}"
    assert np.array_equal(w, w_ref, equal_nan=True), f"ws_nrml differs: {rel(w, w_ref):.3e}"
    assert np.array_equal(r, r_ref, equal_nan=True), f"resid differs: {rel(r, r_ref):.3e}"


@pytest.mark.parametrize("name", ["dirichlet_vortex", "mms"])
def test_residual_dirichlet(name):
    mesh, opt = cases.dirichlet_vortex() if name == "dirichlet_vortex" else cases.mms_box()
    orc = Oracle(mesh, opt)
    orc.initialize_solution()
    r_ref, w_ref = orc.compute_residual(0.37)
    for prec, tol in ((PREC_FP64_STRICT, 1e-13), (PREC_FP64, 1e-12)):
        with Solver(mesh, opt.replace(precision=prec)) as s:
            s.initialize_solution()
            assert np.array_equal(s.cvar, orc.cvar)
            r, w = s.compute_residual(0.37)
        assert rel(r, r_ref) <= tol and rel(w, w_ref) <= tol, (prec, rel(r, r_ref), rel(w, w_ref))


INTEGRATOR_CASES = {
    # (case factory, steps, exact state expected in strict mode)
    "ssprk3_periodic": (lambda: cases.periodic_vortex(16, jitter=0.2), 6, True),
    "rk4_periodic": (lambda: cases.periodic_vortex(16, rk_nstages=4, rk_order=4, ssprk=False, dt_from_cfl=False,
                                                  dt=0.02), 5, True),
    "rk4_order1_periodic": (lambda: cases.periodic_vortex(16, rk_nstages=4, rk_order=1, ssprk=False,
                                                         dt_from_cfl=False, dt=0.005), 4, True),
    "ssprk42_periodic": (lambda: cases.periodic_vortex(16, rk_nstages=4, rk_order=2, ssprk=True,
                                                      dt_from_cfl=False, dt=0.02), 5, True),
    "ssprk42_steady_airfoil": (lambda: cases.airfoil(), 6, True),
    "rk4_steady_airfoil": (lambda: cases.airfoil(ssprk=False, rk_order=4, cfl=0.8), 5, True),
    "ssprk42_dirichlet_vortex": (lambda: cases.dirichlet_vortex(ssprk=True, rk_order=2), 4, False),
    "rk4_dirichlet_vortex": (lambda: cases.dirichlet_vortex(), 4, False),
    "ssprk3_mixed_tri_quad": (lambda: cases.periodic_mixed(14), 5, True),
    "ssprk42_steady_quad_airfoil": (lambda: cases.airfoil_quads(48, 16), 5, True),
    "ssprk42_steady_quad_airfoil_nn": (lambda: cases.airfoil_quads(48, 16, lsq_stencil="nn", limiter=0), 5, True),
}


@pytest.mark.parametrize("name", sorted(INTEGRATOR_CASES))
def test_time_integration(name):
    factory, nsteps, exact = INTEGRATOR_CASES[name]
    mesh, opt = factory()
    orc = Oracle(mesh, opt)
    orc.initialize_solution()
    u0 = orc.cvar
    n_ref = orc.time_integration(0.0, nsteps)
    u_ref = orc.cvar
    with Solver(mesh, opt.replace(precision=PREC_FP64_STRICT)) as s:
        s.cvar = u0
        n = s.time_integration(0.0, nsteps)
        u = s.cvar
    if exact:
        assert np.array_equal(u, u_ref), f"strict state differs: {rel(u, u_ref):.3e}"
    else:
        assert rel(u, u_ref) <= 1e-13, rel(u, u_ref)
    assert np.allclose(n, n_ref, rtol=1e-13, atol=0), (n, n_ref)
    with Solver(mesh, opt.replace(precision=PREC_FP64)) as s:
        s.cvar = u0
        n = s.time_integration(0.0, nsteps)
        assert rel(s.cvar, u_ref) <= 1e-12, rel(s.cvar, u_ref)
        assert np.allclose(n, n_ref, rtol=1e-9), (n, n_ref)


# smooth periodic vortex: 1e-6; transonic airfoil with the Venkatakrishnan
# limiter: FP32 rounding moves limiter values, so the transient differs more
MIXED_TOL = {"ssprk3_periodic": 1e-6, "ssprk42_steady_airfoil": 1e-4}


@pytest.mark.parametrize("name", sorted(MIXED_TOL))
def test_mixed_precision(name):
    factory, nsteps, _ = INTEGRATOR_CASES[name]
    mesh, opt = factory()
    orc = Oracle(mesh, opt)
    orc.initialize_solution()
    u0 = orc.cvar
    orc.time_integration(0.0, nsteps)
    u_ref = orc.cvar
    with Solver(mesh, opt.replace(precision=PREC_MIXED)) as s:
        s.cvar = u0
        s.time_integration(0.0, nsteps)
        u = s.cvar
    err_inf = rel(u, u_ref)
    assert err_inf <= MIXED_TOL[name], err_inf


def test_full_size_residual_bit_exact():
    """Benchmark-size mesh (1024x512 quads -> 1,048,576 cells, jittered,
    periodic): one residual, strict mode, bit-identical to the oracle."""
    mesh, opt = cases.periodic_vortex(1, jitter=0.0)
    from fvs2d_gb300 import meshgen
    mesh = meshgen.periodic_square(1024, 512, jitter=0.2, seed=1, jitter_seed=2)
    orc = Oracle(mesh, opt, nthreads=8)
    orc.initialize_solution()
    r_ref, w_ref = orc.compute_residual(0.0)
    with Solver(mesh, opt.replace(precision=PREC_FP64_STRICT)) as s:
        s.initialize_solution()
        r, w = s.compute_residual(0.0)
        assert s.ncells == 1048576
    assert np.array_equal(r, r_ref), rel(r, r_ref)
    assert np.array_equal(w, w_ref), rel(w, w_ref)


def test_full_size_conservation_and_determinism():
    """Size-independent properties at 1,048,576 cells: the periodic residual
    conserves mass/momentum/energy to round-off, and two runs are identical."""
    from fvs2d_gb300 import meshgen
    mesh = meshgen.periodic_square(1024, 512, jitter=0.2)
    _, opt = cases.periodic_vortex(4)
    with Solver(mesh, opt.replace(precision=PREC_FP64)) as s:
        s.initialize_solution()
        vol = s.export("cell_vol")
        u0 = s.cvar
        tot0 = (vol[:, None] * u0).sum(0)
        s.time_integration(0.0, 3)
        u1 = s.cvar
        s.cvar = u0
        s.time_integration(0.0, 3)
        u2 = s.cvar
    assert np.array_equal(u1, u2)
    tot1 = (vol[:, None] * u1).sum(0)
    assert np.all(np.abs(tot1 - tot0) <= 1e-11 * np.abs(tot0).max()), (tot0, tot1)


def test_nonfinite_detected():
    mesh, opt = cases.periodic_vortex(12)
    with Solver(mesh, opt) as s:
        s.initialize_solution()
        u = s.cvar
        u[5, 0] = np.nan
        s.cvar = u
        with pytest.raises(FvsError) as e:
            s.time_integration(0.0, 2)
        assert e.value.code == capi.FVS_ERR_NONFINITE


def test_nonfinite_detected_without_norm_log():
    """fvs_steps_device asks for no norms; the non-finite state is still
    reported (from the last step's norms on the device)."""
    mesh, opt = cases.periodic_vortex(12)
    with Solver(mesh, opt) as s:
        s.initialize_solution()
        u = s.cvar
        u[7, 2] = np.nan
        s.cvar = u
        with pytest.raises(FvsError) as e:
            s.steps_device(3)
        assert e.value.code == capi.FVS_ERR_NONFINITE


def test_divergence_detected():
    """A time step above the scheme's stability limit: the RMS(dU) of the
    oracle's run (CPU) grows 1.27, 1.70, 2.52, 3.45, 5.38 x the first step's
    and turns non-finite at step 7.  With diverge_factor 2 and a check every
    step, the device run stops with FVS_ERR_DIVERGED at step 4, before any
    value becomes non-finite."""
    mesh, opt = cases.periodic_vortex(24, jitter=0.2, cfl=2.0, diverge_factor=2.0)
    with Solver(mesh, opt) as s:
        s.initialize_solution()
        with pytest.raises(FvsError) as e:
            s.run_to_drop(0.0, 50, drop=1e-10, check_every=1)
        assert e.value.code == capi.FVS_ERR_DIVERGED
        assert np.all(np.isfinite(s.cvar))


def test_run_to_drop_matches_step_log():
    # CFL 0.5: the second-order limited scheme diverges above ~0.8 on this mesh
    mesh, opt = cases.airfoil(nw=64, nr=24, cfl=0.5)
    with Solver(mesh, opt.replace(precision=PREC_FP64_STRICT)) as s:
        s.initialize_solution()
        u0 = s.cvar
        log = s.time_integration(0.0, 60)
        s.cvar = u0
        n, log2 = s.run_to_drop(0.0, 60, drop=0.5, check_every=7)
    want = int(np.argmax(log[:, 0] <= 0.5 * log[0, 0])) + 1 if np.any(log[:, 0] <= 0.5 * log[0, 0]) else 60
    assert n == want
    assert np.array_equal(log2, log[:n])
