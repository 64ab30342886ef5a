"""Accuracy of the arithmetic modes over one vortex period (1,048,576 cells).

The isentropic vortex of the throughput benchmark (periodic [-5,5]^2, 1024x512
quads jittered +-0.2h, seeded diagonals; Mach 0.5 along +x, K = 5; SSP-RK3)
is advected for one period T = 10 / u_inf.  All runs use the same fixed dt:
the CFL-0.8 step of the initial state, shortened so that an integer number of
steps ends exactly at T.  Per gradient method (LSQ-fn, GG-cell, GG-node):

  * the FP64 drop-in: its error against the exact solution
    (error_isentropic_vortex, src/mms.f90:271-365).  The reference's exact
    vortex has no periodic image (its centre is x0 + u_inf t), so it is
    evaluated at t = 0: after one period the exact solution on the periodic
    box is the initial state;
  * the double-float and the mixed modes: L2 and Linf of U - U_fp64 relative
    to max|U_fp64|, and their own errors against the exact solution.
The FP64 drop-in itself is held to the CPU oracle per residual and per step
by the parity tests.
"""
from __future__ import annotations

import json
import math
import time

import numpy as np

from . import PREC_FP64, PREC_FP64_DF, PREC_MIXED, meshgen
from .options import Options
from .solver import Solver

U_INF = 0.5 * math.sqrt(1.4)
PERIOD = 10.0 / U_INF
GRAD_NAMES = {3: "lsq_fn", 1: "gg_cell", 2: "gg_node"}
PREC_NAMES = {PREC_FP64: "fp64", PREC_FP64_DF: "fp64_df", PREC_MIXED: "mixed"}


def vortex_options(grad_method: int, precision: int, dt: float) -> Options:
    return Options(vortex=True, vortex_x=0.0, vortex_y=0.0, vortex_kappa=5.0, vortex_inf=(1.0, U_INF, 0.0, 1.0),
                   grad_method=grad_method, lsq_stencil="fn", lsq_pow=0.0, limiter=0, reconst=2, rk_nstages=3,
                   rk_order=3, ssprk=True, cfl=0.8, dt_from_cfl=False, dt=dt, precision=precision)


def period_dt(mesh) -> tuple[float, int]:
    """The CFL-0.8 dt of the initial state, shortened to T / ceil(T / dt)."""
    o = vortex_options(3, PREC_FP64, 0.0).replace(dt_from_cfl=True)
    with Solver(mesh, o) as s:
        s.initialize_solution()
        s.time_integration(0.0, 1)
        dt_cfl = s.current_dt()
    n = int(math.ceil(PERIOD / dt_cfl))
    return PERIOD / n, n


def _rel(a: np.ndarray, b: np.ndarray) -> tuple[float, float]:
    scale = float(np.abs(b).max())
    d = a - b
    return float(np.abs(d).max() / scale), float(np.sqrt((d * d).mean()) / scale)


def _exact(err13: np.ndarray) -> dict:
    # error_isentropic_vortex: per variable (max, L1, L2), then the total L2
    return {"rho_linf": float(err13[0]), "rho_l2": float(err13[2]), "total_l2": float(err13[12])}


def run(nx=1024, ny=512, methods=(3, 1, 2)) -> dict:
    mesh = meshgen.periodic_square(nx, ny, jitter=0.2, seed=1, jitter_seed=2)
    dt, nsteps = period_dt(mesh)
    out = {"workload": f"isentropic vortex, one period T = {PERIOD:.4f}, {mesh.ncells} cells, SSP-RK3, "
                       f"fixed dt {dt:.6g} ({nsteps} steps, CFL-0.8 step of the initial state shortened to T/n)",
           "errors_vs_fp64": "Linf and L2 of U - U_fp64 relative to max|U_fp64|, after one period",
           "errors_vs_exact": "error_isentropic_vortex against the exact solution at T (= the initial state on the "
                              "periodic box): rho max and L2, total L2", "methods": {}}
    for gm in methods:
        res = {}
        states = {}
        for prec in (PREC_FP64, PREC_FP64_DF, PREC_MIXED):
            with Solver(mesh, vortex_options(gm, prec, dt)) as s:
                s.initialize_solution()
                t0 = time.perf_counter()
                s.time_integration(0.0, nsteps)
                sec = time.perf_counter() - t0
                states[prec] = s.cvar
                res[PREC_NAMES[prec]] = {"vs_exact": _exact(s.error_isentropic_vortex(0.0)),
                                         "seconds": round(sec, 2)}
        for prec in (PREC_FP64_DF, PREC_MIXED):
            linf, l2 = _rel(states[prec], states[PREC_FP64])
            res[PREC_NAMES[prec]]["vs_fp64"] = {"linf": linf, "l2": l2}
        out["methods"][GRAD_NAMES[gm]] = res
    return out


def main(argv=None):
    print(json.dumps(run()), flush=True)


if __name__ == "__main__":
    main()
