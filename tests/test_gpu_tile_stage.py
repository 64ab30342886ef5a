"""The fused RK stages against the separate gradient, flux and update
kernels, for the mixed and double-float precisions, through the C-ABI:
k_tile_stage (one thread block per tile of cells, gradients and face fluxes
kept in shared memory) and k_tile_flux_update (after the gradient kernel,
face fluxes in shared memory and the update, per tile).

Both handles run the same per-cell arithmetic in the same summation order;
only the cell numbering (tiles of compact patches against reverse
Cuthill-McKee) and the blocking of the norm reduction differ.  So states,
residuals and wave-speed sums after n steps are bit-identical, and the
RMS(dU) norms agree to rtol 1e-13 (another order of the blocked sum).
Cases cover every branch of the fused kernel: each gradient (LSQ face and
node neighbours, GG-cell, GG-node), the limiter, UMUSCL, first order, every
integrator (SSP-RK3, SSP-RK(4,2) steady, classic RK4 with Dirichlet ghost
states), meshes of one tile and of many, triangles and quadrilaterals."""
import numpy as np
import pytest

import cases
from fvs2d_gb300 import PREC_FP64_DF, PREC_MIXED, Solver

pytestmark = pytest.mark.gpu

CASES = {
    "vortex_lsq_fn_many_tiles": lambda: cases.periodic_vortex(48, jitter=0.2),
    "vortex_lsq_fn_one_tile": lambda: cases.periodic_vortex(12, jitter=0.2),
    "vortex_lsq_nn": lambda: cases.periodic_vortex(40, jitter=0.2, lsq_stencil="nn", lsq_pow=1.0),
    "vortex_ggcell": lambda: cases.periodic_vortex(40, jitter=0.2, grad_method=1),
    "vortex_ggnode": lambda: cases.periodic_vortex(40, jitter=0.2, grad_method=2),
    "vortex_umuscl": lambda: cases.periodic_vortex(40, jitter=0.2, reconst=3, umuscl=1.0 / 3.0),
    "mixed_cells_ssp3": lambda: cases.periodic_mixed(36),
    "dirichlet_rk4": lambda: cases.dirichlet_vortex(40, 32),
    "airfoil_limited_ssp42": lambda: cases.airfoil(96, 32, cfl=0.5),
    "airfoil_quads_limited": lambda: cases.airfoil_quads(96, 24, cfl=0.5),
    "airfoil_first_order": lambda: cases.airfoil(96, 32, reconst=1),
}


def run(mesh, opt, mode, monkeypatch, steps=6):
    monkeypatch.setenv("FVS2D_TILE_STAGE", str(mode))
    with Solver(mesh, opt) as s:
        s.initialize_solution()
        launches = s.launches_per_step()
        norms = s.time_integration(0.0, steps)
        u = s.cvar
        t = 0.0 if opt.steady else steps * s.current_dt()
        r, w = s.compute_residual(t)
    return launches, norms, u, r, w


@pytest.mark.parametrize("mode", [1, 2, 3])
@pytest.mark.parametrize("prec", [PREC_MIXED, PREC_FP64_DF])
@pytest.mark.parametrize("name", sorted(CASES))
def test_tile_stage_bit_identical_to_separate_kernels(name, prec, mode, monkeypatch):
    """mode 1: the whole stage in one launch per tile (k_tile_stage); mode 2:
    the gradient kernel, then face flux and update in one launch per tile
    (k_tile_flux_update); mode 3: the whole stage per tile with its inputs
    brought into shared memory by bulk copies (k_tile_dma; mixed precision,
    LSQ gradients)."""
    mesh, opt = CASES[name]()
    if mode == 3 and (prec != PREC_MIXED or opt.grad_method != 3):
        pytest.skip("the bulk-copy form covers mixed precision with LSQ gradients")
    opt = opt.replace(precision=prec)
    lf, nf, uf, rf, wf = run(mesh, opt, mode, monkeypatch)
    ls, ns, us, rs, ws = run(mesh, opt, 0, monkeypatch)
    nst = opt.rk_nstages
    grad = 0 if opt.reconst == 1 else 1
    # k_begin_step + per stage one fused launch (mode 1) or gradient + one
    # launch (mode 2)
    assert lf == 1 + nst * (1 if mode in (1, 3) else grad + 1), lf
    assert ls > lf
    assert np.array_equal(uf, us), float(np.abs(uf - us).max())
    assert np.array_equal(rf, rs) and np.array_equal(wf, ws)
    assert np.allclose(nf, ns, rtol=1e-13, atol=0)
