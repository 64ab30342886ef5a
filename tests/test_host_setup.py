"""Host-side preprocessing of the product (fvs_create_host, no GPU) against
the oracle: every connectivity, geometry and stencil array bit-identical,
and the reference's consistency checks returning the same error codes."""
import ctypes as C
import os

import numpy as np
import pytest

import cases
from fvs2d_gb300 import Options, capi, meshgen
from fvs2d_gb300.solver import FLOAT_EXPORTS, INT_EXPORTS
from oracle_lib import Oracle

ALL_EXPORTS = sorted(INT_EXPORTS | FLOAT_EXPORTS)


class HostHandle:
    def __init__(self, mesh, opt):
        self.lib = capi.load()
        self.m = capi.MeshArrays(mesh)
        self.o = opt.to_struct()
        self.h = C.c_void_p()
        self.rc = self.lib.fvs_create_host(C.byref(self.m.struct), C.byref(self.o), C.byref(self.h))
        self.msg = self.lib.fvs_last_error(None).decode()

    def export(self, name):
        n = C.c_int64(0)
        rc = self.lib.fvs_export_size(self.h, name.encode(), C.byref(n))
        if rc:
            return None
        dt = np.int32 if name in INT_EXPORTS else np.float64
        out = np.empty(max(n.value // np.dtype(dt).itemsize, 1), dt)
        if n.value:
            assert self.lib.fvs_export(self.h, name.encode(), capi.ptr(out), n.value) == 0
        return out[: n.value // np.dtype(dt).itemsize]

    def sizes(self):
        s = capi.FvsSizes()
        assert self.lib.fvs_get_sizes(self.h, C.byref(s)) == 0
        return s

    def close(self):
        if self.h:
            self.lib.fvs_destroy(self.h)
            self.h = None


def assert_same_setup(mesh, opt):
    orc = Oracle(mesh, opt)
    hh = HostHandle(mesh, opt)
    assert hh.rc == 0, hh.msg
    try:
        for name in ALL_EXPORTS:
            b = hh.export(name)
            try:
                a = orc.export(name)
            except Exception:
                assert b is None, f"{name}: exported by the product only"
                continue
            assert b is not None, f"{name}: exported by the oracle only"
            assert a.shape == b.shape and np.array_equal(a, b), f"{name} differs"
        so, sp = orc.sizes, hh.sizes()
        for f in ("ncells", "nedges", "nedges_intr", "nedges_bndr", "ncells_intr", "ncells_bndr", "stencil_len",
                  "heff1", "heff2", "vol_sum", "vol_green"):
            assert getattr(so, f) == getattr(sp, f), f
    finally:
        hh.close()


MESHES = {
    "periodic_jitter": lambda: meshgen.periodic_square(18, 14, jitter=0.2),
    "dirichlet_jitter": lambda: meshgen.dirichlet_square(15, 9, jitter=0.2),
    "ogrid": lambda: meshgen.naca0012_ogrid(64, 24),
    "ogrid_bd": lambda: meshgen.naca0012_ogrid(40, 12, diag_ac=False),
    "ogrid_quads": lambda: meshgen.naca0012_ogrid(48, 14, quads=True),
    "periodic_mixed": lambda: meshgen.periodic_square(15, 12, jitter=0.2, quad_every=3),
}
OPTS = {
    "lsq_fn": Options(grad_method=3, lsq_stencil="fn"),
    "lsq_fn_w1": Options(grad_method=3, lsq_stencil="fn", lsq_pow=1.0, limiter=1),
    "lsq_nn": Options(grad_method=3, lsq_stencil="nn", limiter=3),
    "ggcb": Options(grad_method=1),
    "ggnb": Options(grad_method=2),
}


@pytest.mark.parametrize("mesh_name", sorted(MESHES))
@pytest.mark.parametrize("opt_name", sorted(OPTS))
def test_setup_bit_identical(mesh_name, opt_name):
    assert_same_setup(MESHES[mesh_name](), OPTS[opt_name])


def test_mixed_tri_quad_mesh():
    """Quads and triangles in one mesh (quads numbered after triangles)."""
    # a box split into triangles except two middle columns kept as quads
    nx, ny = 6, 5
    w = nx + 1
    xy = np.array([[i * 1.0, j * 1.0] for j in range(ny + 1) for i in range(nx + 1)])
    tris, quads = [], []
    for j in range(ny):
        for i in range(nx):
            a, b, c, d = j * w + i + 1, j * w + i + 2, (j + 1) * w + i + 2, (j + 1) * w + i + 1
            if i in (2, 3) and 0 < j < ny - 1:
                quads.append([a, b, c, d])
            elif (i, j) in ((nx - 1, 0), (0, ny - 1)):
                tris += [[a, b, d], [b, c, d]]  # corner: one boundary edge per cell
            else:
                tris += [[a, b, c], [a, c, d]]
    tris = np.array(tris, np.int32)
    quads = np.array(quads, np.int32)
    # boundary cells: cells owning a box-boundary edge
    allc = [list(t) for t in tris] + [list(q) for q in quads]

    def onb(n):
        x, y = xy[n - 1]
        return x in (0, nx) or y in (0, ny)

    bc = []
    for k, cell in enumerate(allc):
        nv = len(cell)
        for e in range(nv):
            p, q = cell[e], cell[(e + 1) % nv]
            xp, yp = xy[p - 1]
            xq, yq = xy[q - 1]
            if onb(p) and onb(q) and ((xp == xq and xp in (0, nx)) or (yp == yq and yp in (0, ny))):
                bc.append(k + 1)
                break
    mesh = meshgen.Mesh(xy, tris, quads, ["freestream"], [np.array(bc, np.int32)])
    assert_same_setup(mesh, Options(grad_method=3, lsq_stencil="nn"))
    assert_same_setup(mesh, Options(grad_method=2))
    assert_same_setup(mesh, Options(grad_method=1))


def test_reference_example_meshes(reference_examples):
    for sub, stem, opt in (("isentropic_vortex", "vortex", Options(grad_method=3, lsq_stencil="fn")),
                           ("naca0012_ogrid", "naca0012_omesh", Options(grad_method=3, lsq_stencil="nn"))):
        d = os.path.join(reference_examples, sub)
        mesh = meshgen.read_grid(os.path.join(d, stem + ".grid"), os.path.join(d, stem + ".bc"))
        assert_same_setup(mesh, opt)


@pytest.mark.parametrize("case,code", [
    ("two_boundary_edges", capi.FVS_ERR_MESH),
    ("count_mismatch", capi.FVS_ERR_MESH),
    ("solid_wall", capi.FVS_ERR_INVALID),
    ("limiter_with_gg", capi.FVS_ERR_INVALID),
    ("bad_node", capi.FVS_ERR_MESH),
])
def test_errors_match_oracle(case, code):
    mesh = meshgen.dirichlet_square(6, 6)
    opt = Options()
    if case == "two_boundary_edges":
        # a corner triangle with two boundary edges (the reference pairs
        # boundary edge i with boundary cell i)
        mesh = meshgen.dirichlet_square(3, 3)
        t = mesh.tri_nodes
        t[0], t[1] = [1, 2, 5], [2, 6, 5]  # quad (0,0) split along b-d
        cells = set(mesh.bndry_cells[0].tolist()) | {1, 2}
        mesh.bndry_cells = [np.array(sorted(cells), np.int32)]
    elif case == "count_mismatch":
        mesh.bndry_cells = [mesh.bndry_cells[0][1:]]
    elif case == "solid_wall":
        mesh.bndry_types = ["solid_wall"]
    elif case == "limiter_with_gg":
        opt = Options(grad_method=1, limiter=1)
    elif case == "bad_node":
        mesh.tri_nodes[3, 1] = 10**6
    hh = HostHandle(mesh, opt)
    assert hh.rc == code, hh.msg
    assert hh.msg
    with pytest.raises(Exception) as e:
        Oracle(mesh, opt)
    assert getattr(e.value, "code", None) == code


@pytest.mark.parametrize("case,code", [
    ("no_cells", capi.FVS_ERR_INVALID),
    ("no_boundary_list", capi.FVS_ERR_MESH),
    ("degenerate_triangle", capi.FVS_ERR_MESH),
    ("clockwise_triangle", capi.FVS_ERR_MESH),
    ("duplicate_cell", capi.FVS_ERR_MESH),
    ("unused_node", capi.FVS_OK),
])
def test_edge_case_meshes_match_oracle(case, code):
    """Empty and malformed meshes: the library's setup and the oracle give the
    same verdict, and an unused node (allowed by the reference's reader) sets
    up as usual."""
    import copy
    mesh = copy.deepcopy(meshgen.dirichlet_square(6, 6))
    if case == "no_cells":
        mesh.tri_nodes = np.zeros((0, 3), np.int32)
        mesh.bndry_cells = [np.zeros(0, np.int32)]
    elif case == "no_boundary_list":
        mesh.bndry_types, mesh.bndry_cells = [], []
    elif case == "degenerate_triangle":
        mesh.tri_nodes[0, 1] = mesh.tri_nodes[0, 0]
    elif case == "clockwise_triangle":
        mesh.tri_nodes[0] = mesh.tri_nodes[0][::-1]
    elif case == "duplicate_cell":
        mesh.tri_nodes[5] = mesh.tri_nodes[4]
    elif case == "unused_node":
        mesh.node_xy = np.concatenate([mesh.node_xy, [[100.0, 100.0]]])
    hh = HostHandle(mesh, Options())
    try:
        assert hh.rc == code, hh.msg
    finally:
        hh.close()
    if code == capi.FVS_OK:
        Oracle(mesh, Options()).close()
    else:
        with pytest.raises(Exception) as e:
            Oracle(mesh, Options())
        assert getattr(e.value, "code", None) == code
