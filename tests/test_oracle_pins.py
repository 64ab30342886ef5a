"""Pins of the CPU oracle: the reference's own built-in checks (it ships no
golden outputs), run on the oracle.

  - LSQ reproduces grad(2x+y) = (2,1) within 1e-10      src/gradient_lsq.f90:490-529
  - sum of volumes == Green-theorem sum, boundary counts  src/grid_procs.f90:722-728,785-791,824-840
  - MMS truncation error of the residual shrinks with h  src/test.f90:481-519
  - isentropic-vortex error norms stay small             src/mms.f90:271-365
  - LSQ-fn boundary padding = nearest unused cell centres (kd-tree, src/gradient_lsq.f90:85-131)
"""
import numpy as np
import pytest

import cases
from fvs2d_gb300 import Options, meshgen
from oracle_lib import Oracle, OracleError


MESHES = {
    "dirichlet_box": lambda: meshgen.dirichlet_square(14, 11, jitter=0.25),
    "ogrid": lambda: meshgen.naca0012_ogrid(48, 20),
    "periodic": lambda: meshgen.periodic_square(12, 10, jitter=0.2),
}


@pytest.mark.parametrize("mesh_name", sorted(MESHES))
@pytest.mark.parametrize("stencil,pw", [("fn", 0.0), ("nn", 0.0), ("fn", 1.0), ("nn", 2.0)])
def test_lsq_linear_exactness(mesh_name, stencil, pw):
    mesh = MESHES[mesh_name]()
    orc = Oracle(mesh, Options(grad_method=3, lsq_stencil=stencil, lsq_pow=pw))
    xy = orc.export("cell_xy").reshape(-1, 2)
    if mesh.period_x:
        pytest.skip("a linear field is not periodic")
    u = np.zeros((orc.ncells, 4))
    u[:, 0] = 2.0 * xy[:, 0] + xy[:, 1] + 10.0  # rho linear, u = v = 0
    u[:, 3] = 2.5
    orc.cvar = u
    orc.compute_residual(0.0)
    g, _ = orc.gradient()
    assert np.abs(g[0, :, 0] - 2.0).max() < 1e-10
    assert np.abs(g[1, :, 0] - 1.0).max() < 1e-10


@pytest.mark.parametrize("mesh_name", ["dirichlet_box", "ogrid"])
def test_green_identity(mesh_name):
    orc = Oracle(MESHES[mesh_name](), Options())
    s = orc.sizes
    assert abs(s.vol_sum - s.vol_green) <= 1e-12 * abs(s.vol_sum)
    assert s.vol_sum > 0 and s.ncells_bndr == sum(len(c) for c in MESHES[mesh_name]().bndry_cells)


def test_boundary_count_mismatch_rejected():
    mesh = meshgen.dirichlet_square(6, 6)
    mesh.bndry_cells = [mesh.bndry_cells[0][:-1]]
    with pytest.raises(OracleError) as e:
        Oracle(mesh, Options())
    assert e.value.code == 2


def test_mms_truncation_error_decreases():
    """test_resid: L2 of resid + mms_source over interior cells, three meshes."""
    errs, hs = [], []
    for n in (8, 16, 32):
        mesh, opt = cases.mms_box(n, n)
        orc = Oracle(mesh, opt)
        orc.initialize_solution()
        r, _ = orc.compute_residual(0.0)
        src = orc.mms_source()
        intr = orc.export("cell_intr") - 1
        e = r[intr] + src[intr]
        errs.append(np.sqrt((e ** 2).mean(0)))
        hs.append(orc.sizes.heff1)
    errs = np.array(errs)
    # the reference's continuity source uses u*rx where r*ux belongs
    # (src/mms.f90:161), so only momentum and energy converge
    for v in (1, 2, 3):
        assert errs[1, v] < errs[0, v] and errs[2, v] < errs[1, v], errs[:, v]


def test_vortex_error_small():
    mesh, opt = cases.periodic_vortex(32)
    orc = Oracle(mesh, opt)
    orc.initialize_solution()
    e0 = orc.error_isentropic_vortex(0.0)
    assert e0.max() < 1e-5  # periodic images of the vortex only
    orc.time_integration(0.0, 10)
    e = orc.error_isentropic_vortex(10 * orc.dt)
    assert e[0] < 0.05 and e[12] < 0.05, e


@pytest.mark.parametrize("mesh_name", ["dirichlet_box", "ogrid"])
def test_fn_padding_is_nearest(mesh_name):
    """Boundary cells of the LSQ-fn stencil are padded with the nearest cell
    centres that are neither the cell nor a face neighbour."""
    mesh = MESHES[mesh_name]()
    orc = Oracle(mesh, Options(grad_method=3, lsq_stencil="fn"))
    xy = orc.export("cell_xy").reshape(-1, 2)
    nb = orc.export("cell_nghbr").reshape(-1, 4)
    ptr = orc.export("stencil_ptr")
    st = orc.export("stencil_cell")
    checked = 0
    for ic in range(orc.ncells):
        own = nb[ic][nb[ic] >= 0]
        if not np.any(own == 0):
            continue
        d2 = ((xy - xy[ic]) ** 2).sum(1)
        order = np.argsort(d2, kind="stable")[:8] + 1
        pad = [j for j in order if j != ic + 1 and j not in own][: int(np.sum(own == 0))]
        got = [st[k] for k in range(ptr[ic], ptr[ic + 1]) if st[k] not in own[own > 0]]
        assert sorted(pad) == sorted(got), (ic, pad, got)
        checked += 1
    assert checked > 0


def test_parallel_oracle_bit_identical():
    for factory in (lambda: cases.periodic_vortex(16, jitter=0.2), lambda: cases.airfoil(),
                    lambda: cases.dirichlet_vortex()):
        mesh, opt = factory()
        a, b = Oracle(mesh, opt, nthreads=1), Oracle(mesh, opt, nthreads=4)
        a.initialize_solution()
        b.initialize_solution()
        na, nb = a.time_integration(0.0, 3), b.time_integration(0.0, 3)
        assert np.array_equal(a.cvar, b.cvar) and np.array_equal(na, nb)


@pytest.mark.parametrize("bad", [dict(grad_method=1, limiter=1), dict(rk_nstages=3, ssprk=False),
                                 dict(rk_nstages=4, rk_order=3, ssprk=True), dict(flux=2)])
def test_invalid_options_rejected(bad):
    with pytest.raises(OracleError) as e:
        Oracle(meshgen.dirichlet_square(4, 4), Options(**bad))
    assert e.value.code == 1


@pytest.mark.parametrize("grad_method,limiter", [(3, 0), (3, 1), (1, 0), (2, 0)])
def test_free_stream_preserved(grad_method, limiter):
    """Property of the reference's scheme: a uniform state on a closed
    (periodic) mesh has a zero residual up to rounding, with every gradient
    (the faces' normals times lengths of each cell sum to zero)."""
    mesh = meshgen.periodic_square(16, 12, jitter=0.25)
    o = Oracle(mesh, Options(vortex=False, mach_inf=0.6, aoa_inf_deg=20.0, grad_method=grad_method,
                             limiter=limiter, dt=0.01))
    o.initialize_solution()
    u = o.cvar
    assert np.ptp(u, axis=0).max() == 0.0  # a uniform free stream
    r, _ = o.compute_residual(0.0)
    o.close()
    h = 10.0 / 16
    # flux magnitudes are O(1); R = -sum(F.n A)/vol ~ 1/h per unbalanced face
    assert np.abs(r).max() <= 1e-12 / h, np.abs(r).max()


def test_discrete_conservation_periodic():
    """Each interior face's flux leaves one cell and enters the other, so on a
    periodic mesh sum(vol * resid) vanishes to rounding for any state."""
    mesh, opt = cases.periodic_vortex(16, jitter=0.2)
    o = Oracle(mesh, opt)
    o.initialize_solution()
    r, _ = o.compute_residual(0.0)
    vol = mesh_volumes(mesh)
    total = (vol[:, None] * r).sum(axis=0)
    scale = (vol[:, None] * np.abs(r)).sum(axis=0)
    o.close()
    assert np.all(np.abs(total) <= 1e-13 * scale), (total, scale)


def mesh_volumes(mesh):
    """Cell areas from the node coordinates (shoelace), minimum-image across
    the periods, in reference cell order (triangles, then quadrilaterals)."""
    xy = mesh.node_xy
    out = []
    for cells in (mesh.tri_nodes, mesh.quad_nodes):
        if cells.shape[0] == 0:
            continue
        p = xy[cells - 1]  # (n, k, 2)
        d = p - p[:, :1, :]
        if mesh.period_x > 0:
            d[..., 0] -= mesh.period_x * np.round(d[..., 0] / mesh.period_x)
        if mesh.period_y > 0:
            d[..., 1] -= mesh.period_y * np.round(d[..., 1] / mesh.period_y)
        x, y = d[..., 0], d[..., 1]
        out.append(0.5 * (x * np.roll(y, -1, axis=1) - np.roll(x, -1, axis=1) * y).sum(axis=1))
    return np.concatenate(out)
