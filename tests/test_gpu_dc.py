"""Defect-correction iteration of first-order steady batches.

Each chunk evaluates the FP64 residual R0 of the current state once and then
iterates a correction with R0 + J dU, J dU from the FP32 dual-number Roe
flux.  With one step per chunk, a DC step differs from an FP64 RK step only
by the second-order remainder of the linearisation and FP32 rounding of
J dU, so the two trajectories agree to a small fraction of the increments;
a wrong Jacobian term would show at the size of the increments themselves.
Converged, the state is a fixed point of the FP64 iteration.
"""
import numpy as np
import pytest

import cases
from fvs2d_gb300 import PREC_FP64, PREC_MIXED, Solver
from fvs2d_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def first_order_sweep(prec=PREC_MIXED):
    specs = [(48, 16, 0.5, 0.0), (64, 20, 0.7, 1.5), (40, 24, 0.3, -2.0)]
    meshes, opts = [], []
    for nw, nr, mach, aoa in specs:
        m, o = cases.airfoil(nw=nw, nr=nr, mach_inf=mach, aoa_inf_deg=aoa, reconst=1, limiter=0, precision=prec)
        meshes.append(m)
        opts.append(o)
    return meshes, opts


def test_one_step_chunks_follow_the_fp64_trajectory():
    meshes, opts = first_order_sweep(PREC_FP64)
    with Batch(meshes, opts) as b:
        b.initialize_solution()
        b.steps(300)
        start = [b.get_state(c) for c in range(3)]
        b.steps(6)
        ref = [b.get_state(c) for c in range(3)]
        for c in range(3):
            b.set_state(c, start[c])
        never = np.zeros((3, 4))  # levels no case reaches: exactly max_steps steps
        done, first, last, _ = b.run_to_level(6, never, chunk=1, dc=True)
        assert np.all(done == 6)
        got = [b.get_state(c) for c in range(3)]
    for c in range(3):
        inc = np.abs(ref[c] - start[c]).max()
        err = np.abs(got[c] - ref[c]).max()
        assert inc > 0
        assert err <= 1e-3 * inc, (c, err, inc)


def test_tiled_mode_equals_persistent():
    """Defect correction as a graph of tile launches per step: same tile work
    as the persistent kernel, same states to FP32-increment rounding."""
    meshes, opts = first_order_sweep(PREC_MIXED)
    out = []
    for tiled in (False, True):
        with Batch(meshes, opts) as b:
            b.set_mode(tiled, fixed=True)
            b.initialize_solution()
            b.steps(200)
            never = np.zeros((3, 4))
            done, _, last, _ = b.run_to_level(60, never, chunk=25, dc=True)
            assert np.all(done == 60)
            out.append(([b.get_state(c) for c in range(3)], last))
    for c in range(3):
        a, t = out[0][0][c], out[1][0][c]
        assert np.abs(a - t).max() <= 1e-12 * np.abs(a).max(), c
    assert np.allclose(out[0][1], out[1][1], rtol=1e-6, atol=0)


@pytest.mark.parametrize("tiled", [False, True])
def test_fused_stage_matches_separate_phases(tiled):
    """Defect correction with each cell's face J dU inside its stage (one
    phase per stage) against separate J dU and update phases: the same
    corrections up to FP32 rounding, and the same fixed point."""
    meshes, opts = first_order_sweep(PREC_MIXED)
    out = []
    for fused in (False, True):
        with Batch(meshes, opts) as b:
            b.set_mode(tiled, dc_fused=fused, fixed=True)
            b.initialize_solution()
            b.steps(200)
            u0 = [b.get_state(c) for c in range(3)]
            never = np.zeros((3, 4))
            done, _, last, _ = b.run_to_level(60, never, chunk=25, dc=True)
            assert np.all(done == 60)
            out.append(([b.get_state(c) for c in range(3)], last, u0))
    for c in range(3):
        a, t, s0 = out[0][0][c], out[1][0][c], out[0][2][c]
        inc = np.abs(a - s0).max()
        assert np.abs(a - t).max() <= 1e-4 * inc, (c, np.abs(a - t).max(), inc)
    assert np.allclose(out[0][1], out[1][1], rtol=1e-3, atol=0)


def test_shape_trials_keep_results():
    """A defect-correction run tries launch shapes in its first chunks and
    after cases converge; trial chunks are shorter, so the FP64 base state is
    re-evaluated more often, but the run reaches the same fixed point."""
    meshes, opts = first_order_sweep(PREC_MIXED)
    out = []
    for fixed in (True, False):
        with Batch(meshes, opts) as b:
            b.set_mode(False, fixed=fixed)
            b.initialize_solution()
            first, _ = b.steps(1)
            levels = first[:, 0, :] * 1e-9
            b.initialize_solution()
            b.run_to_level(100000, levels * 1e4, chunk=200)
            n2, _, last, _ = b.run_to_level(100000, levels, chunk=200, dc=True)
            assert np.all(n2 < 100000) and np.all(last <= levels)
            out.append([b.get_state(c) for c in range(3)])
    for c in range(3):
        assert np.abs(out[0][c] - out[1][c]).max() <= 1e-6 * np.abs(out[0][c]).max(), c


def test_converges_to_the_fp64_fixed_point():
    meshes, opts = first_order_sweep(PREC_MIXED)
    with Batch(meshes, opts) as b:
        b.initialize_solution()
        first, _ = b.steps(1)
        levels = first[:, 0, :] * 1e-9
        b.initialize_solution()
        n1, _, _, _ = b.run_to_level(100000, levels * 1e4, chunk=200)
        n2, _, last, _ = b.run_to_level(100000, levels, chunk=200, dc=True)
        assert np.all(n2 < 100000)
        assert np.all(last <= levels)
        # the FP64 iteration from the corrected state meets the levels at once
        n3, f3, _, _ = b.run_to_level(1000, levels * 1.5, chunk=10)
        assert np.all(n3 <= 10), n3
        states = [b.get_state(c) for c in range(3)]
    for c in range(3):
        with Solver(meshes[c], opts[c].replace(precision=PREC_FP64)) as s:
            s.initialize_solution()
            r0, _ = s.compute_residual(0.0)
            s.cvar = states[c]
            r, _ = s.compute_residual(0.0)
        assert np.abs(r).max() <= 1e-7 * np.abs(r0).max(), (c, np.abs(r).max(), np.abs(r0).max())


def test_groups_stop_together_and_pick_the_first():
    meshes, opts = first_order_sweep(PREC_MIXED)
    meshes, opts = meshes[:2] + meshes[:2], opts[:2] + opts[:2]
    with Batch(meshes, opts) as b:
        b.initialize_solution()
        first, _ = b.steps(1)
        levels = first[:, 0, :] * 1e-3
        # twins 0/2 and 1/3: case 2 starts from a converged-ish state of case 0
        b.initialize_solution()
        b.run_to_level(100000, levels * 1e-2, chunk=50)
        head = b.get_state(0)
        b.initialize_solution()
        b.set_state(2, head)
        b.set_groups([0, 1, 0, 1])
        done, _, last, _ = b.run_to_level(100000, levels, chunk=7)
        b.set_groups(None)
    # the warm twin met the target and ended the cold one at the same step
    assert done[0] == done[2]
    assert np.all(last[2] <= levels[2])
    assert not np.all(last[0] <= levels[0])
    # identical twins converge on the same step
    assert done[1] == done[3]
    assert np.all(last[1] <= levels[1]) and np.all(last[3] <= levels[3])
