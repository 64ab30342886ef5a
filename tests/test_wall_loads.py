"""Wall pressure coefficient and loads (write_inst_cp_un, src/io.f90:340-446).

CPU: the oracle's restatement against known answers (a uniform free stream
has cp = 0 and no load; a linear pressure field, which the LSQ gradient
reproduces exactly, integrates to the body's area by the divergence theorem).
GPU: fvs_wall_loads against the oracle, bit-exact in strict FP64.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from cases import airfoil, airfoil_quads
from oracle_lib import Oracle

GAMMA = 1.4


def _prim_to_cons(pv):
    u = np.empty_like(pv)
    u[:, 0] = pv[:, 0]
    u[:, 1] = pv[:, 0] * pv[:, 1]
    u[:, 2] = pv[:, 0] * pv[:, 2]
    u[:, 3] = pv[:, 3] / (GAMMA - 1.0) + 0.5 * pv[:, 0] * (pv[:, 1] ** 2 + pv[:, 2] ** 2)
    return u


def _wall_area(mesh, nw):
    x, y = mesh.node_xy[:nw, 0], mesh.node_xy[:nw, 1]
    return 0.5 * abs(np.dot(x, np.roll(y, -1)) - np.dot(y, np.roll(x, -1)))


def test_free_stream_has_no_load():
    mesh, o = airfoil(nw=48, nr=12)
    orc = Oracle(mesh, o)
    orc.initialize_solution()
    n = mesh.bndry_cells[0].size
    e, L = orc.wall_loads(1, n)
    assert np.all(e[:, 1] == 0.0) and np.all(e[:, 2] == 0.0)
    assert L["cl"] == 0.0 and L["cd"] == 0.0
    # |Vn| of the free stream over the wall faces: V_inf . n per face
    a = math.radians(o.aoa_inf_deg)
    eg = orc.export("edge_geom").reshape(-1, 7)
    be = orc.export("bndry_edges")[:n] - 1
    vn = o.mach_inf * (math.cos(a) * eg[be, 3] + math.sin(a) * eg[be, 4])
    assert np.allclose(e[:, 3], vn, rtol=0, atol=1e-14)
    assert L["un_max"] == np.abs(e[:, 3]).max()
    assert L["un_l1"] == pytest.approx(np.abs(vn).mean(), rel=1e-14)
    assert L["un_l2"] == pytest.approx(math.sqrt((vn ** 2).mean()), rel=1e-14)


@pytest.mark.parametrize("reconst", [1, 2])
def test_linear_pressure_integrates_to_body_area(reconst):
    nw = 64
    mesh, o = airfoil(nw=nw, nr=16, reconst=reconst, limiter=0)
    orc = Oracle(mesh, o)
    xy = orc.export("cell_xy").reshape(-1, 2)
    alpha, p0 = 0.3, 1.0 / GAMMA
    pv = np.column_stack([np.ones(len(xy)), np.zeros(len(xy)), np.zeros(len(xy)), p0 + alpha * xy[:, 0]])
    orc.cvar = _prim_to_cons(pv)
    n = mesh.bndry_cells[0].size
    e, L = orc.wall_loads(1, n)
    c2 = 2.0 / o.mach_inf ** 2
    # face pressure is the linear field at the face centre
    eg = orc.export("edge_geom").reshape(-1, 7)
    be = orc.export("bndry_edges")[:n] - 1
    assert np.allclose(e[:, 1], c2 * alpha * (eg[be, 0] - 0.0) + c2 * (p0 - 1.0 / GAMMA), atol=1e-11)
    # sum cp n_x A = c2 alpha * (closed integral of x n_x) = -+ c2 alpha * area
    area = _wall_area(mesh, nw)
    assert abs(L["ca"]) == pytest.approx(c2 * alpha * area, rel=1e-10)
    assert abs(L["cn"]) < 1e-10


def test_rejects_non_wall_boundary():
    mesh, o = airfoil(nw=32, nr=8)
    orc = Oracle(mesh, o)
    orc.initialize_solution()
    from oracle_lib import OracleError
    with pytest.raises(OracleError):
        orc.wall_loads(2, 4)  # boundary 2 is the far field
    with pytest.raises(OracleError):
        orc.wall_loads(3, 4)


def _perturbed(orc, seed):
    rng = np.random.default_rng(seed)
    u = orc.cvar
    u *= 1.0 + 0.02 * rng.standard_normal(u.shape)
    return u


@pytest.mark.gpu
@pytest.mark.parametrize("reconst,grad,quads", [(2, 3, False), (1, 3, False), (2, 1, False), (2, 2, False),
                                                (2, 3, True), (2, 2, True)])
def test_gpu_wall_loads_bit_exact(reconst, grad, quads):
    from fvs2d_gb300 import PREC_FP64_STRICT, Solver
    factory = airfoil_quads if quads else airfoil
    mesh, o = factory(nw=64, nr=20, reconst=reconst, grad_method=grad, limiter=1 if grad == 3 else 0,
                      precision=PREC_FP64_STRICT)
    orc = Oracle(mesh, o)
    orc.initialize_solution()
    orc.time_integration(0.0, 3)
    u = _perturbed(orc, 11)
    orc.cvar = u
    n = mesh.bndry_cells[0].size
    e0, L0 = orc.wall_loads(1, n)
    with Solver(mesh, o) as s:
        s.cvar = u
        e1, L1 = s.wall_loads(1)
    assert np.array_equal(e0, e1)
    for k in ("cn", "ca", "cn1", "ca1", "un_max", "un_l2", "un_l1", "cl", "cd", "cl1", "cd1"):
        assert L0[k] == L1[k], k


@pytest.mark.gpu
def test_gpu_wall_loads_fp64_and_mixed_tolerance(tmp_path):
    from fvs2d_gb300 import PREC_FP64, PREC_MIXED, Solver
    mesh, o = airfoil(nw=64, nr=20)
    orc = Oracle(mesh, o)
    orc.initialize_solution()
    orc.time_integration(0.0, 5)
    u = orc.cvar
    _, L0 = orc.wall_loads(1, mesh.bndry_cells[0].size)
    for prec, tol in ((PREC_FP64, 1e-12), (PREC_MIXED, 1e-5)):
        with Solver(mesh, o.replace(precision=prec)) as s:
            s.cvar = u
            _, L1 = s.wall_loads(1)
            loads = s.write_cp(str(tmp_path / "cp.plt"))
        assert abs(L1["cl"] - L0["cl"]) <= tol * max(1.0, abs(L0["cl"]))
        assert abs(L1["cd"] - L0["cd"]) <= tol * max(1.0, abs(L0["cd"]))
        assert loads["cl"] == L1["cl"]
    lines = (tmp_path / "cp.plt").read_text().splitlines()
    assert lines[0] == 'TITLE     = "cp"' and lines[2] == f"ZONE I={mesh.bndry_cells[0].size} J=1"
    assert len(lines) == 4 + mesh.bndry_cells[0].size
