"""Writes tests/golden/reference_examples.npz from the reference's own example
inputs, so that the GPU parity tests can run them where the reference
sources are not mounted.

The reference ships two cases, each a mesh (.grid, .bc), a scheme file
(fvs2d.input) and, for the vortex, its parameters (fvs2d.vortex):

  examples/isentropic_vortex   7,226 triangles, Dirichlet exact-vortex
                               boundary, LSQ face neighbours, classic 4-stage
                               RK of order 4, dt 0.01 (unsteady)
  examples/naca0012_ogrid      65,536 quadrilaterals, slip wall + free
                               stream, LSQ node neighbours, SSP-RK(4,2) with
                               local time steps at CFL 1.25 (steady)

Per case the fixture holds the mesh exactly as meshgen.read_grid parses it,
the options as options.read_input parses the two scheme files (JSON), and
the oracle's run of STEPS steps from initialize_solution: the RMS(dU) norms
of every step, and SHA-256 digests of the final state and of
compute_residual there (resid, ws_nrml), computed on the machine that wrote
the fixture.  The digests pin the oracle's arithmetic on that machine
(tests/test_reference_examples.py); the GPU tests compare against the oracle
run live on the GPU host.

    FVS2D_REFERENCE=<reference checkout> python tests/golden/make_reference_examples.py
"""
from __future__ import annotations

import dataclasses
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from fvs2d_gb300 import Options, meshgen  # noqa: E402
from fvs2d_gb300.options import read_input  # noqa: E402

STEPS = 20
OUT = os.path.join(HERE, "reference_examples.npz")
# case name -> (example directory, grid base name)
EXAMPLES = {"isentropic_vortex": ("isentropic_vortex", "vortex"),
            "naca0012_ogrid": ("naca0012_ogrid", "naca0012_omesh")}


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a, np.float64).tobytes())
    return h.hexdigest()


def read_example(reference_dir: str, name: str):
    """(mesh, options) of one example, read with the library's parsers."""
    sub, stem = EXAMPLES[name]
    d = os.path.join(reference_dir, "examples", sub)
    mesh = meshgen.read_grid(os.path.join(d, stem + ".grid"), os.path.join(d, stem + ".bc"))
    opt = read_input(os.path.join(d, "fvs2d.input"))
    return mesh, opt


def pack(name: str, mesh, opt) -> dict:
    p = name + "/"
    return {p + "node_xy": np.asarray(mesh.node_xy, np.float64),
            p + "tri_nodes": np.asarray(mesh.tri_nodes, np.int32).reshape(-1, 3),
            p + "quad_nodes": np.asarray(mesh.quad_nodes, np.int32).reshape(-1, 4),
            p + "bndry_types": np.array(mesh.bndry_types),
            p + "bndry_counts": np.array([len(c) for c in mesh.bndry_cells], np.int32),
            p + "bndry_cells": np.concatenate([np.asarray(c, np.int32) for c in mesh.bndry_cells]),
            p + "options": np.array(json.dumps(dataclasses.asdict(opt)))}


def unpack(z, name: str):
    """(mesh, options) of one case from the loaded fixture."""
    p = name + "/"
    counts = z[p + "bndry_counts"]
    cells = np.split(z[p + "bndry_cells"], np.cumsum(counts)[:-1])
    mesh = meshgen.Mesh(z[p + "node_xy"].copy(), z[p + "tri_nodes"].copy(), z[p + "quad_nodes"].copy(),
                        [str(t) for t in z[p + "bndry_types"]], [np.asarray(c, np.int32) for c in cells],
                        0.0, 0.0, name)
    o = json.loads(str(z[p + "options"]))
    o["vortex_inf"] = tuple(o["vortex_inf"])
    return mesh, Options(**o)


def oracle_run(mesh, opt, nthreads: int = 1) -> dict:
    """STEPS steps of the oracle from initialize_solution: the start state,
    norms, final state and compute_residual at the final time."""
    from oracle_lib import Oracle
    o = Oracle(mesh, opt, nthreads=nthreads)
    try:
        o.initialize_solution()
        start = o.cvar
        norms = o.time_integration(0.0, STEPS)
        state = o.cvar
        t_end = 0.0 if opt.steady else STEPS * o.dt
        resid, ws = o.compute_residual(t_end)
        # magnitude of the face fluxes the residual sums, per unit volume:
        # sum over faces of 0.5 (|un| + a) A, over vol, times max|U|
        vol = o.export("cell_vol")
        flux_scale = float(np.max(ws / vol * np.abs(state).max(axis=1)))
        return dict(start=start, norms=norms, state=state, resid=resid, ws=ws, t_end=t_end, flux_scale=flux_scale)
    finally:
        o.close()


def main():
    ref = os.environ.get("FVS2D_REFERENCE", "/root/reference")
    out = {}
    for name in EXAMPLES:
        mesh, opt = read_example(ref, name)
        out.update(pack(name, mesh, opt))
        r = oracle_run(mesh, opt, nthreads=os.cpu_count() or 1)
        out[name + "/norms"] = r["norms"]
        out[name + "/digest_state"] = np.array(digest(r["state"]))
        out[name + "/digest_residual"] = np.array(digest(r["resid"], r["ws"]))
        print(name, mesh.ncells, "cells")
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
