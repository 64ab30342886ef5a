"""Synthetic meshes in the reference's .grid/.bc data model.

Every generator returns a :class:`Mesh` holding exactly what ``grid_read`` and
``grid_bc_read`` load (src/grid_procs.f90:65-164): node coordinates, triangle
and quad node lists (1-based, counter-clockwise), and per-boundary cell lists
with a type string.  Randomness comes from a splitmix64 stream with a fixed
seed, so every mesh is reproducible bit-for-bit on any machine.

Meshes:
  * :func:`periodic_square` -- the isentropic-vortex box, each quad split along
    a seeded random diagonal, optional seeded node jitter; doubly periodic
    (an extension: the reference has no periodic boundary).
  * :func:`dirichlet_square` -- the same box with one Dirichlet boundary, as in
    the reference's vortex example; corner quads are split so that no cell has
    two boundary edges (the reference pairs boundary edge i with boundary cell
    i, src/residual.f90:114-125).
  * :func:`naca0012_ogrid` -- an O-grid around a closed-trailing-edge NACA0012:
    cosine-clustered wall nodes, rays from the mid-chord point, geometric
    radial stretching with a given first spacing, far field at a given radius,
    quads split along a fixed diagonal; boundary 1 = slip_wall, 2 = freestream.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

BC_CODES = {"freestream": 1, "slip_wall": 2, "solid_wall": 3, "dirichlet": 4}

_MASK = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n outputs of the splitmix64 generator started at ``seed`` (uint64)."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = (np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)) & _MASK
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _MASK
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _MASK
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, n: int) -> np.ndarray:
    """n doubles in [0,1) from the top 53 bits of splitmix64(seed)."""
    return (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclasses.dataclass
class Mesh:
    node_xy: np.ndarray            # (nnodes, 2) float64
    tri_nodes: np.ndarray          # (ntri, 3) int32, 1-based
    quad_nodes: np.ndarray         # (nquad, 4) int32, 1-based
    bndry_types: list              # type strings, one per boundary
    bndry_cells: list              # int32 arrays of 1-based cell ids
    period_x: float = 0.0
    period_y: float = 0.0
    name: str = "mesh"

    @property
    def nnodes(self) -> int:
        return int(self.node_xy.shape[0])

    @property
    def ncells(self) -> int:
        return int(self.tri_nodes.shape[0] + self.quad_nodes.shape[0])


def _split_quads(a, b, c, d, diag_ac):
    """Two CCW triangles per CCW quad (a,b,c,d): diagonal a-c or b-d."""
    t1 = np.where(diag_ac[:, None], np.stack([a, b, c], 1), np.stack([a, b, d], 1))
    t2 = np.where(diag_ac[:, None], np.stack([a, c, d], 1), np.stack([b, c, d], 1))
    tris = np.empty((2 * a.shape[0], 3), dtype=np.int32)
    tris[0::2] = t1
    tris[1::2] = t2
    return tris


def periodic_square(nx: int, ny: int, x0: float = -5.0, y0: float = -5.0, lx: float = 10.0,
                    ly: float = 10.0, seed: int = 1, jitter: float = 0.0, jitter_seed: int = 2,
                    quad_every: int = 0) -> Mesh:
    """Doubly periodic box of nx*ny quads, 2*nx*ny triangles.

    Node (i,j) has id j*nx+i+1; the nodes at x0+lx / y0+ly are the ones at
    x0 / y0.  ``jitter`` displaces every node by a seeded uniform amount in
    [-jitter*h, +jitter*h] per axis.  ``quad_every`` > 0 keeps the quads of
    every column i with i % quad_every == 0 (a mixed triangle/quad mesh;
    cells are numbered triangles first, then quads)."""
    hx, hy = lx / nx, ly / ny
    i = np.arange(nx)
    j = np.arange(ny)
    X = (x0 + hx * i)[None, :].repeat(ny, 0)
    Y = (y0 + hy * j)[:, None].repeat(nx, 1)
    xy = np.stack([X.ravel(), Y.ravel()], 1).astype(np.float64)
    if jitter > 0.0:
        r = uniform01(jitter_seed, 2 * nx * ny).reshape(-1, 2)
        xy[:, 0] += (2.0 * r[:, 0] - 1.0) * jitter * hx
        xy[:, 1] += (2.0 * r[:, 1] - 1.0) * jitter * hy
    I, J = np.meshgrid(i, j)
    I = I.ravel()
    J = J.ravel()
    ip = (I + 1) % nx
    jp = (J + 1) % ny
    a = (J * nx + I + 1).astype(np.int32)
    b = (J * nx + ip + 1).astype(np.int32)
    c = (jp * nx + ip + 1).astype(np.int32)
    d = (jp * nx + I + 1).astype(np.int32)
    diag = (splitmix64(seed, nx * ny) & np.uint64(1)).astype(bool)
    if quad_every > 0:
        keep = (I % quad_every) == 0
        tris = _split_quads(a[~keep], b[~keep], c[~keep], d[~keep], diag[~keep])
        quads = np.stack([a[keep], b[keep], c[keep], d[keep]], 1).astype(np.int32)
        return Mesh(xy, tris, quads, [], [], lx, ly, f"periodic_mixed_{nx}x{ny}")
    tris = _split_quads(a, b, c, d, diag)
    return Mesh(xy, tris, np.zeros((0, 4), np.int32), [], [], lx, ly, f"periodic_{nx}x{ny}")


def dirichlet_square(nx: int, ny: int, x0: float = -5.0, y0: float = -5.0, lx: float = 10.0,
                     ly: float = 10.0, seed: int = 1, jitter: float = 0.0, jitter_seed: int = 2,
                     bc: str = "dirichlet") -> Mesh:
    """Box of nx*ny quads with one boundary of type ``bc`` around it."""
    hx, hy = lx / nx, ly / ny
    i = np.arange(nx + 1)
    j = np.arange(ny + 1)
    X = (x0 + hx * i)[None, :].repeat(ny + 1, 0)
    Y = (y0 + hy * j)[:, None].repeat(nx + 1, 1)
    xy = np.stack([X.ravel(), Y.ravel()], 1).astype(np.float64)
    if jitter > 0.0:
        r = uniform01(jitter_seed, 2 * (nx + 1) * (ny + 1)).reshape(-1, 2)
        ii, jj = np.meshgrid(i, j)
        inner = ((ii > 0) & (ii < nx) & (jj > 0) & (jj < ny)).ravel()
        xy[inner, 0] += ((2.0 * r[:, 0] - 1.0) * jitter * hx)[inner]
        xy[inner, 1] += ((2.0 * r[:, 1] - 1.0) * jitter * hy)[inner]
    qi, qj = np.meshgrid(np.arange(nx), np.arange(ny))
    qi = qi.ravel()
    qj = qj.ravel()
    w = nx + 1
    a = (qj * w + qi + 1).astype(np.int32)
    b = (qj * w + qi + 2).astype(np.int32)
    c = ((qj + 1) * w + qi + 2).astype(np.int32)
    d = ((qj + 1) * w + qi + 1).astype(np.int32)
    diag = (splitmix64(seed, nx * ny) & np.uint64(1)).astype(bool)
    # corner quads: bottom-left / top-right need a-c, bottom-right / top-left b-d
    diag[(qi == 0) & (qj == 0)] = True
    diag[(qi == nx - 1) & (qj == ny - 1)] = True
    diag[(qi == nx - 1) & (qj == 0)] = False
    diag[(qi == 0) & (qj == ny - 1)] = False
    tris = _split_quads(a, b, c, d, diag)
    # boundary cells: triangles owning an edge on the box boundary
    on_b = np.zeros(xy.shape[0] + 1, bool)
    ii, jj = np.meshgrid(i, j)
    on_b[1:] = ((ii == 0) | (ii == nx) | (jj == 0) | (jj == ny)).ravel()
    cells = []
    for k in range(3):
        n1 = tris[:, k]
        n2 = tris[:, (k + 1) % 3]
        # an edge lies on the boundary iff both nodes do and they share a side
        x1, y1 = xy[n1 - 1, 0], xy[n1 - 1, 1]
        x2, y2 = xy[n2 - 1, 0], xy[n2 - 1, 1]
        ia1 = np.rint((x1 - x0) / hx)
        ia2 = np.rint((x2 - x0) / hx)
        ja1 = np.rint((y1 - y0) / hy)
        ja2 = np.rint((y2 - y0) / hy)
        side = ((ia1 == ia2) & ((ia1 == 0) | (ia1 == nx))) | ((ja1 == ja2) & ((ja1 == 0) | (ja1 == ny)))
        cells.append(on_b[n1] & on_b[n2] & side)
    isb = cells[0] | cells[1] | cells[2]
    nbe = cells[0].astype(int) + cells[1] + cells[2]
    assert nbe.max() <= 1, "a cell with two boundary edges"
    bcells = (np.nonzero(isb)[0] + 1).astype(np.int32)
    return Mesh(xy, tris, np.zeros((0, 4), np.int32), [bc], [bcells], 0.0, 0.0, f"{bc}_{nx}x{ny}")


def naca0012_thickness(x: np.ndarray) -> np.ndarray:
    """NACA 4-digit half thickness for t=0.12 with the closed trailing edge
    coefficient (-0.1036)."""
    x = np.clip(x, 0.0, 1.0)
    return 0.6 * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x**2 + 0.2843 * x**3 - 0.1036 * x**4)


def _geometric_ratio(d1: np.ndarray, total: np.ndarray, n: int) -> np.ndarray:
    """q with d1*(q^n-1)/(q-1) = total, per ray (bisection, vectorised)."""
    lo = np.full_like(total, 1.0 + 1e-12)
    hi = np.full_like(total, 2.0)
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        s = d1 * (mid**n - 1.0) / (mid - 1.0)
        big = s > total
        hi = np.where(big, mid, hi)
        lo = np.where(big, lo, mid)
    return 0.5 * (lo + hi)


def naca0012_ogrid(nw: int = 512, nr: int = 256, first: float = 1.0e-3, far: float = 20.0,
                   center=(0.5, 0.0), diag_ac: bool = True, quads: bool = False) -> Mesh:
    """O-grid with nw wall nodes and nr radial nodes, 2*nw*(nr-1) triangles
    (``quads``: nw*(nr-1) quadrilaterals, like the reference's own example).

    Node (i,k) (i around the wall, k outward) has id k*nw+i+1."""
    s = 2.0 * math.pi * np.arange(nw) / nw
    xw = 0.5 * (1.0 + np.cos(s))
    yw = naca0012_thickness(xw) * np.where(s <= math.pi, 1.0, -1.0)
    xw[0], yw[0] = 1.0, 0.0
    cx, cy = center
    th = np.arctan2(yw - cy, xw - cx)
    xf = cx + far * np.cos(th)
    yf = cy + far * np.sin(th)
    dist = np.hypot(xf - xw, yf - yw)
    q = _geometric_ratio(np.full(nw, first), dist, nr - 1)
    k = np.arange(nr)[:, None]
    rho = first * (q[None, :] ** k - 1.0) / (q[None, :] - 1.0)
    rho[-1, :] = dist
    ux = (xf - xw) / dist
    uy = (yf - yw) / dist
    X = xw[None, :] + rho * ux[None, :]
    Y = yw[None, :] + rho * uy[None, :]
    xy = np.stack([X.ravel(), Y.ravel()], 1).astype(np.float64)
    qi, qk = np.meshgrid(np.arange(nw), np.arange(nr - 1))
    qi = qi.ravel()
    qk = qk.ravel()
    ip = (qi + 1) % nw
    # (i,k) -> (i,k+1) -> (i+1,k+1) -> (i+1,k) is counter-clockwise for a
    # counter-clockwise wall parametrisation with outward k
    a = (qk * nw + qi + 1).astype(np.int32)
    b = ((qk + 1) * nw + qi + 1).astype(np.int32)
    c = ((qk + 1) * nw + ip + 1).astype(np.int32)
    d = (qk * nw + ip + 1).astype(np.int32)
    if quads:
        # cell q+1 is quad q = (qk, qi); wall cells k = 0, far cells k = nr-2,
        # both in wall-node order
        qq = np.stack([a, b, c, d], 1).astype(np.int32)
        wall = (np.nonzero(qk == 0)[0] + 1).astype(np.int32)
        farc = (np.nonzero(qk == nr - 2)[0] + 1).astype(np.int32)
        return Mesh(xy, np.zeros((0, 3), np.int32), qq, ["slip_wall", "freestream"], [wall, farc], 0.0, 0.0,
                    f"naca0012_quad_{nw}x{nr}")
    tris = _split_quads(a, b, c, d, np.full(a.shape[0], diag_ac))
    # wall cells: the triangle holding edge d-a (k=0); far cells: edge b-c (k=nr-2)
    ncell = tris.shape[0]
    wall, farc = [], []
    for t in range(2):
        cell_ids = np.arange(t, ncell, 2)
        tri = tris[cell_ids]
        qq = cell_ids // 2
        kk = qk[qq]
        onwall = (kk == 0) & ((tri <= nw).sum(1) == 2)
        onfar = (kk == nr - 2) & ((tri > (nr - 1) * nw).sum(1) == 2)
        wall.append(np.stack([qi[qq][onwall], cell_ids[onwall]], 1))
        farc.append(np.stack([qi[qq][onfar], cell_ids[onfar]], 1))
    wall = np.concatenate(wall)
    farc = np.concatenate(farc)
    wall = wall[np.argsort(wall[:, 0], kind="stable")][:, 1] + 1
    farc = farc[np.argsort(farc[:, 0], kind="stable")][:, 1] + 1
    return Mesh(xy, tris, np.zeros((0, 4), np.int32), ["slip_wall", "freestream"],
                [wall.astype(np.int32), farc.astype(np.int32)], 0.0, 0.0, f"naca0012_{nw}x{nr}")


def signed_areas(mesh: Mesh) -> np.ndarray:
    t = mesh.tri_nodes - 1
    x = mesh.node_xy[:, 0]
    y = mesh.node_xy[:, 1]
    if mesh.period_x > 0 or mesh.period_y > 0:
        def unw(v, ref, L):
            return v - L * np.rint((v - ref) / L) if L > 0 else v
        x1, y1 = x[t[:, 0]], y[t[:, 0]]
        x2, y2 = unw(x[t[:, 1]], x1, mesh.period_x), unw(y[t[:, 1]], y1, mesh.period_y)
        x3, y3 = unw(x[t[:, 2]], x1, mesh.period_x), unw(y[t[:, 2]], y1, mesh.period_y)
    else:
        x1, x2, x3 = x[t[:, 0]], x[t[:, 1]], x[t[:, 2]]
        y1, y2, y3 = y[t[:, 0]], y[t[:, 1]], y[t[:, 2]]
    return 0.5 * (x1 * (y2 - y3) + x2 * (y3 - y1) + x3 * (y1 - y2))


# --------------------------------------------------------------------------
# reference file formats (src/grid_procs.f90:65-164)
# --------------------------------------------------------------------------
def write_grid(mesh: Mesh, grid_path: str, bc_path: str) -> None:
    """Write .grid / .bc files readable by the reference (%.17g coordinates)."""
    with open(grid_path, "w") as f:
        f.write(" #nodes, #cells_tri, #cells_quad\n")
        f.write(f" {mesh.nnodes} {mesh.tri_nodes.shape[0]} {mesh.quad_nodes.shape[0]}\n")
        np.savetxt(f, mesh.node_xy, fmt="%.17g")
        np.savetxt(f, mesh.tri_nodes, fmt="%d")
        if mesh.quad_nodes.shape[0]:
            np.savetxt(f, mesh.quad_nodes, fmt="%d")
    with open(bc_path, "w") as f:
        f.write(f"{len(mesh.bndry_types)}   !-- #boundaries\n")
        for t, c in zip(mesh.bndry_types, mesh.bndry_cells):
            f.write(f"{len(c)}   {t}\n")
        for c in mesh.bndry_cells:
            np.savetxt(f, np.asarray(c).reshape(-1, 1), fmt="%d")


def _fortran_float(tok: str) -> float:
    return float(tok.replace("d", "e").replace("D", "e"))


def read_grid(grid_path: str, bc_path: str) -> Mesh:
    """Read reference .grid / .bc files (list-directed, one record per line)."""
    with open(grid_path) as f:
        f.readline()
        nn, nt, nq = (int(t) for t in f.readline().split()[:3])
        xy = np.array([[_fortran_float(t) for t in f.readline().split()[:2]] for _ in range(nn)], np.float64)
        tri = np.array([[int(t) for t in f.readline().split()[:3]] for _ in range(nt)], np.int32).reshape(-1, 3)
        quad = np.array([[int(t) for t in f.readline().split()[:4]] for _ in range(nq)], np.int32).reshape(-1, 4)
    types, counts, cells = [], [], []
    with open(bc_path) as f:
        nb = int(f.readline().split()[0])
        for _ in range(nb):
            tok = f.readline().split()
            counts.append(int(tok[0]))
            types.append(tok[1])
        for ib in range(nb):
            cells.append(np.array([int(f.readline().split()[0]) for _ in range(counts[ib])], np.int32))
    return Mesh(xy, tri, quad, types, cells, 0.0, 0.0, grid_path)
