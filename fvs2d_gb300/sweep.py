"""Seeded airfoil sweeps and the plain / batched drivers that run them.

The sweep distribution: NACA0012 O-grids with W wall nodes ~ U{wall} and R
radial nodes ~ U{radial}, Mach ~ U[mach], angle of attack ~ U[aoa] degrees,
all drawn from splitmix64(seed).  Each case is steady: local time stepping
with SSP-RK(4,2) (the reference's steady example integrator,
src/runge_kutta.f90:349-418).

Convergence: the reference's second-order limited scheme stalls on these
meshes (its Venkatakrishnan limiter, src/gradient_limiter.f90:113-117, keeps
switching; the RMS(dU) plateaus near 0.1-0.2 of its first value), so the
time-to-drop runs use its first-order reconstruction (face_reconst 1,
src/input.f90:246-248), which converges.  The drop is measured against a
fixed per-case reference level, the first-step residual of a free-stream
start, so that a warm start is judged on the same absolute threshold.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

from . import capi, meshgen
from .options import Options


@dataclasses.dataclass
class Case:
    nw: int
    nr: int
    mach: float
    aoa: float

    def mesh(self) -> meshgen.Mesh:
        return meshgen.naca0012_ogrid(self.nw, self.nr)


def draw_cases(ncases: int, seed: int, wall=(64, 512), radial=(32, 256), mach=(0.3, 0.85), aoa=(-2.0, 4.0)):
    u = meshgen.uniform01(seed, 4 * ncases).reshape(ncases, 4)
    out = []
    for k in range(ncases):
        nw = int(wall[0] + np.floor(u[k, 0] * (wall[1] - wall[0] + 1)))
        nr = int(radial[0] + np.floor(u[k, 1] * (radial[1] - radial[0] + 1)))
        nw += nw % 2  # even wall count: node 0 is the trailing edge, node nw/2 the leading edge
        out.append(Case(nw, nr, mach[0] + u[k, 2] * (mach[1] - mach[0]), aoa[0] + u[k, 3] * (aoa[1] - aoa[0])))
    return out


def case_options(c: Case, precision: int, first_order: bool = True) -> Options:
    return Options(mach_inf=c.mach, aoa_inf_deg=c.aoa, steady=True, cfl=1.25 if first_order else 0.5, rk_nstages=4,
                   rk_order=2, ssprk=True, grad_method=3, lsq_stencil="fn", limiter=1,
                   reconst=1 if first_order else 2, dt=0.01, precision=precision)


def wall_distance(mesh: meshgen.Mesh, nw: int, xy: np.ndarray, k: int = 8) -> np.ndarray:
    """Distance from points to the wall polygon (nodes 1..nw of the O-grid):
    the smallest distance to the segments on either side of the point's k
    nearest wall nodes (a k-d tree query).  The nearest point of the polygon
    lies on such a segment unless a segment longer than the distance between
    k consecutive nodes passes closer; for the O-grid walls, whose nodes
    follow the profile smoothly, this is the exact polygon distance."""
    from scipy.spatial import cKDTree
    w = mesh.node_xy[:nw]
    k = min(k, nw)
    _, idx = cKDTree(w).query(xy, k=k)
    idx = idx.reshape(xy.shape[0], k)
    seg = np.concatenate([idx, (idx - 1) % nw], axis=1)  # segment s runs from node s to node s+1
    a = w[seg]
    ab = w[(seg + 1) % nw] - a
    t = ((xy[:, None, :] - a) * ab).sum(-1) / np.maximum((ab * ab).sum(-1), 1e-300)
    t = np.clip(t, 0.0, 1.0)
    p = a + t[..., None] * ab
    return np.sqrt(((xy[:, None, :] - p) ** 2).sum(-1)).min(1)


def free_stream_state(c: Case, ncells: int, gamma: float = 1.4) -> np.ndarray:
    a = np.deg2rad(c.aoa)
    rho, u, v, p = 1.0, c.mach * np.cos(a), c.mach * np.sin(a), 1.0 / gamma
    e = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)
    return np.tile(np.array([rho, rho * u, rho * v, e]), (ncells, 1))


def free_stream_state_like(o, like: np.ndarray) -> np.ndarray:
    """Free-stream state of options o with the shape of `like`."""
    return free_stream_state(Case(0, 0, o.mach_inf, o.aoa_inf_deg), like.shape[0], o.gamma)


def run_plain(cases, precision, max_steps, drop, starts=None, ref_levels=None, check_every=200, states=None,
              meshes=None):
    """One Solver per case, one after the other (the plain path).  Returns
    per-case steps, wall seconds total (mesh generation excluded when meshes
    are given), and the first-step residuals; the final states are appended
    to `states` when a list is given."""
    from .solver import Solver
    steps, firsts = [], []
    meshes = meshes if meshes is not None else [None] * len(cases)
    t0 = time.perf_counter()
    for k, c in enumerate(cases):
        with Solver(meshes[k] if meshes[k] is not None else c.mesh(), case_options(c, precision)) as s:
            s.initialize_solution()
            if starts is not None:
                s.cvar = starts[k]
            n, log = _run_absolute(s, max_steps, drop, ref_levels[k] if ref_levels is not None else None, check_every)
            steps.append(n)
            firsts.append(log[0])
            if states is not None:
                states.append(s.cvar)
    return np.array(steps), time.perf_counter() - t0, np.array(firsts)


def _run_absolute(s, max_steps, drop, ref_level, check_every):
    """Steps until RMS(dU_k) <= drop * ref_level[k] in all four components
    (ref_level None: the first step's norms)."""
    logs, done = [], 0
    first = None if ref_level is None else np.broadcast_to(np.asarray(ref_level, np.float64), (4,))
    while done < max_steps:
        n = min(check_every, max_steps - done)
        log = s.time_integration(0.0, n)
        logs.append(log)
        if first is None:
            first = log[0].copy()
        hit = np.nonzero(np.all(log <= drop * first[None, :], axis=1))[0]
        if hit.size:
            done += int(hit[0]) + 1
            logs[-1] = log[: int(hit[0]) + 1]
            break
        done += n
    return done, np.concatenate(logs)
