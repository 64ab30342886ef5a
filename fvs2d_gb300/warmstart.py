"""Learned warm start for airfoil sweeps.

A network maps per-cell features (Mach, angle of attack, the cell centroid
x, y and the wall distance) to the converged conservative state; the solver
starts from its prediction instead of the free stream and still iterates to
the same absolute residual threshold, so the network only changes how many
steps are needed, never the answer.  Training data are converged solutions
the solver itself produces; training and inference run on the GPU
(fvs2d_gb300.mlp).

The fast solve is the precision ladder on a batch: mixed precision until
each case's RMS(dU) reaches `switch` x its reference levels in every
component (the FP32 flux floor lies near 5e-6 of them), then FP64 to `drop`
x the reference levels.
"""
from __future__ import annotations

import time

import numpy as np

from . import PREC_FP64, PREC_MIXED, sweep
from .batch import Batch
from .mlp import MLP

N_FEATURES = 5


def cell_centroids(mesh) -> np.ndarray:
    t = mesh.tri_nodes - 1
    return mesh.node_xy[t].mean(1)


def features(case: sweep.Case, mesh) -> np.ndarray:
    xy = cell_centroids(mesh)
    d = sweep.wall_distance(mesh, case.nw, xy)
    r = np.hypot(xy[:, 0] - 0.5, xy[:, 1])
    f = np.empty((xy.shape[0], N_FEATURES), np.float32)
    f[:, 0] = (case.mach - 0.575) / 0.16
    f[:, 1] = (case.aoa - 1.0) / 1.75
    f[:, 2] = (xy[:, 0] - 0.5) / (0.5 + r)
    f[:, 3] = xy[:, 1] / (0.5 + r)
    f[:, 4] = np.log10(d + 1e-4) / 2.0
    return f


def targets(case: sweep.Case, cvar: np.ndarray) -> np.ndarray:
    return (cvar - sweep.free_stream_state(case, cvar.shape[0])).astype(np.float32)


def solve_ladder_raced(meshes, opts_mixed, levels, starts, **kw):
    """The ladder with every case started twice, from `starts` and from the
    free stream, in one batch; the twin that reaches the final level first
    ends its group (the free stream is the fallback of a poor prediction).
    Returns (states, steps_mixed, steps after the switch, seconds, phases,
    winner) with winner[c] = 0 for the given start, 1 for the free stream."""
    n = len(meshes)
    lv = np.asarray(levels, np.float64).reshape(n, 4)
    fs = [sweep.free_stream_state_like(o, u) for o, u in zip(opts_mixed, starts)]
    states, n1, n2, secs, phases, done_last = solve_ladder(
        list(meshes) + list(meshes), list(opts_mixed) + list(opts_mixed), np.concatenate([lv, lv]),
        starts=list(starts) + fs, groups=list(range(n)) * 2, _return_last=True, **kw)
    last = done_last
    ok = np.all(last <= np.concatenate([lv, lv]) * kw.get("drop", 1e-10) * (1 + 1e-12), axis=1)
    tot = n1 + n2
    winner = np.zeros(n, np.int32)
    for c in range(n):
        a, b = (ok[c], tot[c]), (ok[c + n], tot[c + n])
        if b[0] and (not a[0] or b[1] < a[1]):
            winner[c] = 1
    pick = [states[c + n * winner[c]] for c in range(n)]
    return (pick, np.array([n1[c + n * winner[c]] for c in range(n)]),
            np.array([n2[c + n * winner[c]] for c in range(n)]), secs, phases, winner)


def solve_ladder(meshes, opts_mixed, levels, switch=1e-5, drop=1e-10, max_steps=200000, chunk=200, starts=None,
                 autotune=True, dc=True, groups=None, _return_last=False):
    """Batched precision-ladder solve to levels*drop (levels: per-case
    reference residuals [ncases][4]): mixed precision to levels*switch, then
    (dc) the defect-correction iteration to levels*drop followed by the FP64
    iteration, which confirms the levels, or (not dc) FP64 alone.  Returns
    (states, steps_mixed, steps after the switch, seconds, phase seconds)."""
    t0 = time.perf_counter()
    phases = {}
    with Batch(meshes, opts_mixed) as b:
        b.initialize_solution()
        if starts is not None:
            for c, u in enumerate(starts):
                b.set_state(c, u)
        t1 = time.perf_counter()
        phases["setup"] = t1 - t0
        if autotune:
            b.autotune(10)
        t2 = time.perf_counter()
        phases["tune"] = t2 - t1
        n1, _, _, _ = b.run_to_level(max_steps, np.asarray(levels) * switch, chunk)
        t3 = time.perf_counter()
        phases["mixed"] = t3 - t2
        n2 = np.zeros_like(n1)
        if groups is not None:
            b.set_groups(groups)
        if dc:
            n2, _, _, _ = b.run_to_level(max_steps, np.asarray(levels) * drop, chunk, dc=True)
            t4 = time.perf_counter()
            phases["dc"] = t4 - t3
            t3 = t4
        b.set_precision(PREC_FP64)
        n3, _, last, _ = b.run_to_level(max_steps, np.asarray(levels) * drop, 10 if dc else chunk)
        n2 = n2 + n3
        phases["fp64"] = time.perf_counter() - t3
        states = [b.get_state(c) for c in range(b.ncases)]
    if _return_last:
        return states, n1, n2, time.perf_counter() - t0, phases, last
    return states, n1, n2, time.perf_counter() - t0, phases


def reference_levels(cases, meshes):
    """First-step RMS(dU) per component of a free-stream start (the plain
    path's first residuals), [ncases][4], one FP64 batch step."""
    with Batch(meshes, [sweep.case_options(c, PREC_FP64) for c in cases]) as b:
        b.initialize_solution()
        norms, _ = b.steps(1)
    return norms[:, 0, :].copy()


class WarmStart:
    def __init__(self, width=256, depth=4, seed=0):
        self.net = MLP(N_FEATURES, width, depth, 4, seed=seed)
        self.scale = np.ones(4, np.float32)

    def fit(self, X, Y, epochs=20, batch=4096, lr=1e-3, seed=0):
        self.scale = np.maximum(Y.std(0), 1e-6).astype(np.float32)
        return self.net.train(X, Y / self.scale, batch=batch, epochs=epochs, lr=lr, seed=seed)

    def predict_state(self, case: sweep.Case, mesh, feats: np.ndarray | None = None) -> np.ndarray:
        """The predicted conservative state of a case (feats: its features,
        when already computed)."""
        f = features(case, mesh) if feats is None else feats
        dU = self.net.predict(f) * self.scale
        u = sweep.free_stream_state(case, f.shape[0]) + dU.astype(np.float64)
        # keep the state physical (positive density and pressure)
        u[:, 0] = np.maximum(u[:, 0], 0.05)
        ke = 0.5 * (u[:, 1] ** 2 + u[:, 2] ** 2) / u[:, 0]
        u[:, 3] = np.maximum(u[:, 3], ke + 0.05 / 0.4)
        return u


def build_dataset(cases, states, max_cells_per_case=20000, seed=0, feats=None):
    """Training samples: per case at most max_cells_per_case cells (seeded
    draw) of (features, converged state minus free stream); feats: the
    cases' features when already computed."""
    rng = np.random.default_rng(seed)
    X, Y = [], []
    for k, (c, u) in enumerate(zip(cases, states)):
        f = features(c, c.mesh()) if feats is None else feats[k]
        t = targets(c, u)
        if f.shape[0] > max_cells_per_case:
            sel = rng.choice(f.shape[0], max_cells_per_case, replace=False)
            f, t = f[sel], t[sel]
        X.append(f)
        Y.append(t)
    return np.concatenate(X), np.concatenate(Y)
