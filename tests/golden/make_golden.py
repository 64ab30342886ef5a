"""Writes the golden fixtures of tests/golden/ from the CPU oracle.

The reference ships no golden outputs and cannot be built here (no Fortran
compiler, no MPI), so these fixtures are outputs of the oracle, the C
restatement of the reference that tests/test_oracle_pins.py holds to the
reference's own known-answer checks.  Committed, they pin the oracle against
later edits and give the GPU tests fixed numbers to meet.

Per case: the mesh's node coordinates (the generators call numpy's
trigonometric functions, whose last bit differs between platforms), the
start state (the free stream or the initial vortex of initialize_solution),
the state after STEPS RK steps from it, the RMS(dU) norms of those steps and
compute_residual (resid and ws_nrml) at the final state, all in reference
cell order.

    python tests/golden/make_golden.py        # rewrites tests/golden/*.npz
"""
from __future__ import annotations

import copy
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import cases  # noqa: E402
from oracle_lib import Oracle  # noqa: E402

STEPS = 12


def golden_cases():
    """name -> (mesh, options); use with_nodes() to put a fixture's node
    coordinates into the mesh"""
    out = {}
    out["airfoil_lsq_venkat"] = cases.airfoil(32, 10)
    out["airfoil_quads_lsq_nn"] = cases.airfoil_quads(24, 8, lsq_stencil="nn")
    # the smooth vortex with each gradient (Green-Gauss runs without a
    # limiter: the reference's limiter needs the LSQ stencil)
    for gname, gm in (("lsq", 3), ("ggcell", 1), ("ggnode", 2)):
        out[f"periodic_vortex_ssprk3_{gname}"] = cases.periodic_vortex(12, jitter=0.2, grad_method=gm)
    return out


def with_nodes(mesh, node_xy):
    """The mesh with the given node coordinates (connectivity unchanged)."""
    m = copy.deepcopy(mesh)
    assert m.node_xy.shape == node_xy.shape
    m.node_xy = np.array(node_xy, np.float64)
    return m


def compute(mesh, opt):
    o = Oracle(mesh, opt)
    try:
        o.initialize_solution()
        start = o.cvar
        norms = o.time_integration(0.0, STEPS)
        state = o.cvar
        t_end = 0.0 if opt.steady else STEPS * o.dt
        resid, ws = o.compute_residual(t_end)
        return dict(node_xy=np.asarray(mesh.node_xy, np.float64), start=start, norms=norms, state=state, resid=resid,
                    ws=ws, t_end=np.array(t_end))
    finally:
        o.close()


def main():
    for name, (mesh, opt) in golden_cases().items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **compute(mesh, opt))
        print(name, mesh.ncells, "cells")


if __name__ == "__main__":
    main()
