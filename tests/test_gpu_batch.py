"""Batched persistent path vs the single-mesh path, through the C-ABI.

Every per-cell and per-edge computation of the persistent kernel is the same
device code as the three-kernel path.  In the strict FP64 build (no FMA
contraction) each case of a batch equals a single-mesh run bit-for-bit; with
contraction allowed the compiler may fuse different multiply-adds in the two
kernels, so FP64 agrees to 1e-13 and mixed to 1e-6 of max|U|.  Norms come
from a different blocking (rtol 1e-13 in FP64).
"""
import numpy as np
import pytest

import cases
from fvs2d_gb300 import PREC_FP64, PREC_FP64_STRICT, PREC_MIXED, FvsError, Solver, capi
from fvs2d_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def sweep(n=3, prec=PREC_MIXED, **kw):
    specs = [(48, 16, 0.5, 0.0), (64, 20, 0.75, 1.5), (40, 24, 0.3, -2.0)][:n]
    meshes, opts = [], []
    for nw, nr, mach, aoa in specs:
        m, o = cases.airfoil(nw=nw, nr=nr, cfl=0.5, mach_inf=mach, aoa_inf_deg=aoa, precision=prec, **kw)
        meshes.append(m)
        opts.append(o)
    return meshes, opts


STATE_TOL = {PREC_FP64_STRICT: 0.0, PREC_FP64: 1e-13, PREC_MIXED: 1e-6}


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("prec", [PREC_FP64_STRICT, PREC_FP64, PREC_MIXED])
def test_batch_equals_single_mesh_runs(prec):
    meshes, opts = sweep(prec=prec)
    nsteps = 7
    with Batch(meshes, opts) as b:
        b.initialize_solution()
        norms, _ = b.steps(nsteps)
        got = [b.get_state(c) for c in range(b.ncases)]
    for c, (m, o) in enumerate(zip(meshes, opts)):
        with Solver(m, o) as s:
            s.initialize_solution()
            ref_norms = s.time_integration(0.0, nsteps)
            ref = s.cvar
        if prec == PREC_FP64_STRICT:
            assert np.array_equal(got[c], ref), (c, rel(got[c], ref))
        else:
            assert rel(got[c], ref) <= STATE_TOL[prec], (c, rel(got[c], ref))
        assert np.allclose(norms[c], ref_norms, rtol=1e-5 if prec == PREC_MIXED else 1e-12, atol=0)


@pytest.mark.parametrize("first_order", [False, True])
def test_batch_mixed_cell_types_strict(first_order):
    """A quadrilateral O-grid and a triangular one in one batch, strict FP64:
    each case bit-identical to its single-mesh run (second and first order)."""
    kw = dict(reconst=1, limiter=0) if first_order else {}
    m1, o1 = cases.airfoil_quads(40, 14, cfl=0.5, precision=PREC_FP64_STRICT, **kw)
    m2, o2 = cases.airfoil(48, 16, cfl=0.5, mach_inf=0.6, aoa_inf_deg=2.0, precision=PREC_FP64_STRICT, **kw)
    with Batch([m1, m2], [o1, o2]) as b:
        b.initialize_solution()
        b.steps(6)
        got = [b.get_state(c) for c in range(2)]
    for c, (m, o) in enumerate(((m1, o1), (m2, o2))):
        with Solver(m, o) as s:
            s.initialize_solution()
            s.time_integration(0.0, 6)
            assert np.array_equal(got[c], s.cvar), (c, rel(got[c], s.cvar))


def test_batch_unsteady_periodic_strict():
    m1, o1 = cases.periodic_vortex(16, jitter=0.2, dt_from_cfl=False, dt=0.05, precision=PREC_FP64_STRICT)
    m2, o2 = cases.periodic_vortex(24, jitter=0.1, dt_from_cfl=False, dt=0.05, precision=PREC_FP64_STRICT)
    starts = []
    for m, o in ((m1, o1), (m2, o2)):
        with Solver(m, o) as s:
            s.initialize_solution()
            starts.append(s.cvar)
    with Batch([m1, m2], [o1, o2]) as b:
        for c in range(2):
            b.set_state(c, starts[c])
        b.steps(5)
        got = [b.get_state(0), b.get_state(1)]
    for g, (m, o) in zip(got, [(m1, o1), (m2, o2)]):
        with Solver(m, o) as s:
            s.initialize_solution()
            s.time_integration(0.0, 5)
            assert np.array_equal(g, s.cvar)


@pytest.mark.parametrize("first_order", [False, True])
def test_barrier_timeout_reported_and_recoverable(first_order):
    """A zero wait budget makes every grid-barrier wait run out (second- and
    first-order persistent kernels): the kernel returns, the call reports
    FVS_ERR_TIMEOUT, and the batch still works."""
    meshes, opts = sweep(2, **(dict(reconst=1, limiter=0) if first_order else {}))
    with Batch(meshes, opts) as b:
        b.initialize_solution()
        b.set_barrier_budget(0.0)
        with pytest.raises(FvsError) as e:
            b.steps(2)
        assert e.value.code == capi.FVS_ERR_TIMEOUT
        b.set_barrier_budget(4.0)
        b.initialize_solution()
        norms, _ = b.steps(3)
        assert np.isfinite(norms).all()


@pytest.mark.parametrize("prec,first_order", [(PREC_FP64_STRICT, False), (PREC_FP64_STRICT, True),
                                               (PREC_MIXED, False)])
def test_tiled_mode_equals_persistent(prec, first_order):
    """A graph of per-phase tile launches runs the tile work of the persistent
    kernel in the same order: strict FP64 states and norms bit-identical, over
    two chunks (the device step counter restarts from the host's)."""
    meshes, opts = sweep(prec=prec, **(dict(reconst=1, limiter=0) if first_order else {}))
    res = []
    for tiled in (False, True):
        with Batch(meshes, opts) as b:
            b.set_mode(tiled)
            b.initialize_solution()
            n1, _ = b.steps(5)
            n2, _ = b.steps(3)
            assert b.info()["tiled"] == tiled
            res.append((np.concatenate([n1, n2], axis=1), [b.get_state(c) for c in range(len(meshes))]))
    (np_, up), (nt, ut) = res
    for c in range(len(meshes)):
        if prec == PREC_FP64_STRICT:
            assert np.array_equal(ut[c], up[c]), (c, rel(ut[c], up[c]))
        else:
            assert rel(ut[c], up[c]) <= STATE_TOL[prec], (c, rel(ut[c], up[c]))
    if prec == PREC_FP64_STRICT:
        assert np.array_equal(nt, np_)
    else:
        assert np.allclose(nt, np_, rtol=1e-5, atol=0)


@pytest.mark.parametrize("tiled", [False, True])
def test_fused_first_order_stage_matches_separate_phases(tiled):
    """First-order mixed batches evaluate each cell's face fluxes inside its
    stage (one phase per stage).  Same flux and summation order as the
    separate edge-flux and update phases: states agree to FP32 rounding of
    the increments; the second-order batch is never fused."""
    meshes, opts = sweep(prec=PREC_MIXED, reconst=1, limiter=0)
    res = []
    for fused in (False, True):
        with Batch(meshes, opts) as b:
            b.set_mode(tiled, fused=fused)
            b.initialize_solution()
            n1, _ = b.steps(40)
            assert b.info()["fused"] == fused
            res.append((n1, [b.get_state(c) for c in range(3)]))
    for c in range(3):
        assert rel(res[1][1][c], res[0][1][c]) <= 1e-6, (c, rel(res[1][1][c], res[0][1][c]))
    assert np.allclose(res[1][0], res[0][0], rtol=1e-4, atol=0)
    m2, o2 = sweep(1, prec=PREC_MIXED)
    with Batch(m2, o2) as b:
        b.initialize_solution()
        b.steps(1)
        assert not b.info()["fused"]


def test_shape_trials_keep_results():
    """run_to_level tries other launch shapes (fused or not, tiled or not,
    other tiles) once cases converge; every shape runs the same per-cell
    arithmetic, so the steps each case takes and its state equal those of a
    fixed shape.  A converged case stops at the end of its chunk, so both
    runs use chunks of the trial length (20 steps)."""
    meshes, opts = sweep(prec=PREC_MIXED, reconst=1, limiter=0)
    out = []
    for fixed in (True, False):
        with Batch(meshes, opts) as b:
            b.set_mode(False, fixed=fixed)
            b.initialize_solution()
            first, _ = b.steps(1)
            b.initialize_solution()
            levels = first[:, 0, :] * np.array([1e-1, 1e-2, 1e-3])[:, None]
            done, _, _, _ = b.run_to_level(20000, levels, chunk=20)
            assert np.all(done < 20000)
            out.append((done, [b.get_state(c) for c in range(3)]))
    assert np.array_equal(out[0][0], out[1][0]), (out[0][0], out[1][0])
    for c in range(3):
        assert rel(out[1][1][c], out[0][1][c]) <= 1e-6, (c, rel(out[1][1][c], out[0][1][c]))


def test_autotune_keeps_state_and_results():
    meshes, opts = sweep(3)
    with Batch(meshes, opts) as b:
        b.initialize_solution()
        u0 = [b.get_state(c) for c in range(3)]
        ms = b.autotune(2)
        assert ms > 0
        info = b.info()
        assert info["block"] in (128, 256) and info["tile"] >= info["block"]
        for c in range(3):
            assert np.array_equal(b.get_state(c), u0[c])
        n1, _ = b.steps(4)
        b.set_launch(256, 1024, 1)
        b.initialize_solution()
        n2, _ = b.steps(4)
    assert np.allclose(n1, n2, rtol=1e-9)


def test_run_to_drop_per_case():
    meshes, opts = sweep(3)
    with Batch(meshes, opts) as b:
        b.initialize_solution()
        log, _ = b.steps(80)
        b.initialize_solution()
        done, first, last, _ = b.run_to_drop(80, drop=0.3, chunk=9)
    for c in range(3):
        hit = np.nonzero(np.all(log[c] <= 0.3 * log[c, 0][None, :], axis=1))[0]
        want = int(hit[0]) + 1 if hit.size else 80
        assert done[c] == want, (c, done[c], want)
        assert np.allclose(first[c], log[c, 0], rtol=1e-12)
