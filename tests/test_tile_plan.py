"""Tile plans of the fused RK stages, checked on the CPU (no GPU): every
index the fused kernels derive from the plan (local cells, stencil
entries, faces, gather entries) lies within the shared-memory extents and
device arrays it indexes (fvs_tile_plan_info runs check_tile_plan), every
bulk copy of the bulk-copy form starts on a 16-byte boundary with a multiple
of 16 bytes and stays within its array (check_tile_dma), and the shared
memory of the largest tile stays within a block's limit."""
import ctypes as C
import os

import numpy as np
import pytest

import cases
from fvs2d_gb300 import capi, meshgen

# the library's tile size (FVS2D_TILE_CELLS overrides the default of 512)
TILE_CELLS = int(os.environ.get("FVS2D_TILE_CELLS", "512"))
SMEM_OPTIN = 232448  # bytes of shared memory one GB300 block may opt in to


def plan(mesh, opt):
    lib = capi.load()
    m = capi.MeshArrays(mesh)
    o = opt.to_struct()
    info = np.zeros(8, np.int32)
    rc = lib.fvs_tile_plan_info(C.byref(m.struct), C.byref(o), capi.ptr(info))
    assert rc == capi.FVS_OK, lib.fvs_last_error(None).decode()
    return info


CASES = {
    "vortex_fn_one_tile": lambda: cases.periodic_vortex(12, jitter=0.2),
    "vortex_fn": lambda: cases.periodic_vortex(48, jitter=0.2),
    "vortex_nn": lambda: cases.periodic_vortex(48, jitter=0.2, lsq_stencil="nn"),
    "vortex_ggcell": lambda: cases.periodic_vortex(48, jitter=0.2, grad_method=1),
    "vortex_ggnode": lambda: cases.periodic_vortex(48, jitter=0.2, grad_method=2),
    "mixed_cells": lambda: cases.periodic_mixed(36),
    "dirichlet": lambda: cases.dirichlet_vortex(40, 32),
    "airfoil": lambda: cases.airfoil(96, 32),
    "airfoil_quads_nn": lambda: cases.airfoil_quads(96, 24, lsq_stencil="nn"),
    "vortex_1m_cells": lambda: cases.periodic_vortex(1, jitter=0.0),  # replaced below
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_tile_plan_indices_within_bounds(name):
    if name == "vortex_1m_cells":
        mesh = meshgen.periodic_square(1024, 512, jitter=0.2, seed=1, jitter_seed=2)
        opt = cases.periodic_vortex(4)[1]
    else:
        mesh, opt = CASES[name]()
    ntiles, lmax, gmax, fmax, ok, nhalo, dma_smem, dma_ok = plan(mesh, opt)
    assert ok == 1 and dma_ok == 1
    # the bulk-copy form's block (mixed) fits a block's shared memory
    assert dma_smem <= SMEM_OPTIN, dma_smem
    assert ntiles >= 1 and ntiles <= -(-mesh.ncells // (TILE_CELLS // 2))
    assert gmax <= lmax
    # shared memory of one tile block in the double-float build (8-byte
    # values: the larger of the two fused builds) plus the static norm buffer
    assert 8 * (4 * lmax + 9 * gmax + 5 * fmax) + 8 * 1024 + 64 <= SMEM_OPTIN, (lmax, gmax, fmax)
    # compact tiles: the halos are a fraction of the cells
    if ntiles > 8 and TILE_CELLS >= 512:
        assert nhalo < 0.8 * mesh.ncells, nhalo
