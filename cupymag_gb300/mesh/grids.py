"""Meshes: structured periodic hex grid and tetrahedral .nas meshes.

Host-side setup, same conventions as the reference:

* HexGrid (cupymag/mesh/gridHex.py:22-213): nodes i-major / k-fastest,
  node_id(i,j,k) = i(Ny+1)(Nz+1) + j(Nz+1) + k; element corner order of
  gridHex.py:119-126; defect elements have their centre in [c - Nd/2, c + Nd/2)
  on every axis (gridHex.py:98-139).  The periodic DOF map has the closed
  form dof = (i mod Nx) Ny Nz + (j mod Ny) Nz + (k mod Nz), which is what the
  reference's first-appearance dictionary loop produces (gridHex.py:179-213).
* TetraGrid (cupymag/mesh/gridTet.py:26-225): GRID/CTETRA cards of a
  free-field (comma separated) Nastran file, node ids mapped through a sorted
  search; defect flag by element centroid; periodic map that wraps the maximum
  coordinate onto the minimum, rounds to 12 decimals and numbers keys in
  first-appearance order -- here vectorised with np.unique.
"""
from __future__ import annotations

import numpy as np

from ..utils.defect_shapes import get_defect_shape_function


class HexGrid:
    def __init__(self, Nx, Ny, Nz, Ndx, Ndy, Ndz, defect_center=None):
        self.Nx, self.Ny, self.Nz = int(Nx), int(Ny), int(Nz)
        self.Ndx, self.Ndy, self.Ndz = Ndx, Ndy, Ndz
        self.defect_center = defect_center
        self.x = np.linspace(0, Nx, Nx + 1)
        self.y = np.linspace(0, Ny, Ny + 1)
        self.z = np.linspace(0, Nz, Nz + 1)

    def node_id(self, i, j, k):
        return (i * (self.Ny + 1) + j) * (self.Nz + 1) + k

    def defect_bounds(self):
        if self.defect_center is None:
            c = (self.Nx / 2.0, self.Ny / 2.0, self.Nz / 2.0)
        else:
            c = tuple(float(v) for v in self.defect_center)
        d = (self.Ndx, self.Ndy, self.Ndz)
        return [(c[a] - d[a] / 2.0, c[a] + d[a] / 2.0) for a in range(3)]

    def defect_cells(self):
        """Boolean (Nx,Ny,Nz) array: cell (i,j,k) is non-magnetic."""
        b = self.defect_bounds()
        ax = []
        for a, N in enumerate((self.Nx, self.Ny, self.Nz)):
            ctr = np.arange(N) + 0.5
            ax.append((ctr >= b[a][0]) & (ctr < b[a][1]))
        return ax[0][:, None, None] & ax[1][None, :, None] & ax[2][None, None, :]

    def std_fem_mesh(self):
        Nx, Ny, Nz = self.Nx, self.Ny, self.Nz
        i3, j3, k3 = np.meshgrid(np.arange(Nx + 1), np.arange(Ny + 1), np.arange(Nz + 1), indexing="ij")
        coords = np.stack((self.x[i3.ravel()], self.y[j3.ravel()], self.z[k3.ravel()]), axis=1)
        ei, ej, ek = (a.ravel() for a in np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing="ij"))
        el = np.empty((Nx * Ny * Nz, 9), dtype=np.int32)
        for col, (di, dj, dk) in enumerate(((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
                                            (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1))):
            el[:, col] = self.node_id(ei + di, ej + dj, ek + dk)
        el[:, 8] = self.defect_cells().ravel().astype(np.int32)
        return coords, el

    def build_periodic_node_map(self, node_coords=None):
        Nx, Ny, Nz = self.Nx, self.Ny, self.Nz
        i, j, k = np.meshgrid(np.arange(Nx + 1), np.arange(Ny + 1), np.arange(Nz + 1), indexing="ij")
        return ((i % Nx) * (Ny * Nz) + (j % Ny) * Nz + (k % Nz)).ravel().astype(np.int32)

    def defect_dofs(self):
        """Sorted DOF ids of all corners of defect cells (final_assembly.py:27-57)."""
        cells = self.defect_cells()
        if not cells.any():
            return np.zeros(0, dtype=np.int32)
        Nx, Ny, Nz = self.Nx, self.Ny, self.Nz
        mark = np.zeros((Nx, Ny, Nz), dtype=bool)
        for di in (0, 1):
            for dj in (0, 1):
                for dk in (0, 1):
                    mark |= np.roll(np.roll(np.roll(cells, di, 0), dj, 1), dk, 2)
        return np.flatnonzero(mark.ravel()).astype(np.int32)


def read_nas(path):
    """GRID and CTETRA cards of a free-field Nastran file (gridTet.py:88-152)."""
    grids, tets = [], []
    with open(path) as fh:
        for raw in fh:
            if raw.startswith("$") or raw.isspace():
                continue
            if raw.lstrip().startswith("ENDDATA"):
                break
            line = raw.rstrip()
            if line.startswith("GRID"):
                f = [c.strip() for c in line.split(",")]
                grids.append((int(f[1]), float(f[3]), float(f[4]), float(f[5])))
            elif line.startswith("CTETRA"):
                f = [c.strip() for c in line.split(",")]
                tets.append((int(f[1]), int(f[3]), int(f[4]), int(f[5]), int(f[6])))
    if not grids or not tets:
        raise ValueError("File contains no GRID or CTETRA cards")
    g = np.array(grids, dtype=np.float64)
    t = np.array(tets, dtype=np.int64)
    node_ids = g[:, 0].astype(np.int32)
    coords = g[:, 1:4].copy()
    order = np.argsort(node_ids, kind="stable")
    elem_nodes = order[np.searchsorted(node_ids[order], t[:, 1:5], side="left")]
    return node_ids, coords, t[:, 0].astype(np.int32), elem_nodes


def write_nas(path, coords, tets):
    """Write GRID/CTETRA cards (1-based ids) in free-field format."""
    with open(path, "w") as f:
        f.write("$ cupymag_gb300 tetrahedral mesh\n")
        for i, c in enumerate(coords):
            f.write(f"GRID,{i + 1},,{float(c[0])!r},{float(c[1])!r},{float(c[2])!r}\n")
        for e, t in enumerate(tets):
            f.write(f"CTETRA,{e + 1},1,{t[0] + 1},{t[1] + 1},{t[2] + 1},{t[3] + 1}\n")
        f.write("ENDDATA\n")


class TetraGrid:
    def __init__(self, nas_filename=None, defect_shape=None, defect_center=None, coords=None, tets=None):
        if coords is None:
            _, coords, _, tets = read_nas(nas_filename)
        self.node_coords = np.asarray(coords, dtype=np.float64)
        self.element_nodes = np.asarray(tets, dtype=np.int64)
        self.defect_shape = defect_shape
        if defect_center is None:
            defect_center = (self.node_coords.min(axis=0) + self.node_coords.max(axis=0)) / 2
        self.defect_center = np.asarray(defect_center, dtype=np.float64)

    def std_fem_mesh(self):
        el = np.zeros((len(self.element_nodes), 5), dtype=np.int32)
        el[:, :4] = self.element_nodes
        centers = self.node_coords[self.element_nodes].mean(axis=1)
        if self.defect_shape is not None:
            el[:, 4] = np.asarray(self.defect_shape(centers - self.defect_center)).astype(np.int32)
        return self.node_coords, el

    def build_periodic_node_map(self, node_coords=None, tol=1e-12):
        c = self.node_coords if node_coords is None else np.asarray(node_coords)
        lo, hi = c.min(axis=0), c.max(axis=0)
        w = np.where(np.abs(c - hi[None, :]) < tol, lo[None, :], c)
        keys = np.round(w, 12)
        _, first, inv = np.unique(keys, axis=0, return_index=True, return_inverse=True)
        rank = np.empty(len(first), dtype=np.int64)
        rank[np.argsort(first, kind="stable")] = np.arange(len(first))
        return rank[inv.ravel()].astype(np.int32)


def kuhn_tet_cube(ne, jitter=0.0, seed=0, edge=None):
    """A cube of ne^3 cells split into 6 Kuhn tetrahedra each.

    Interior nodes are jittered uniformly by +-jitter*h (seeded); boundary
    nodes stay on the faces so the periodic map pairs them.  Each tet is
    ordered so that its signed Jacobian is positive.  Edge length defaults to
    ne (h = 1, the reference's length unit).
    """
    h = 1.0 if edge is None else edge / ne
    rng = np.random.default_rng(seed)
    g = np.arange(ne + 1, dtype=np.float64)
    I, J, K = np.meshgrid(g, g, g, indexing="ij")
    coords = np.stack([I.ravel(), J.ravel(), K.ravel()], axis=1)
    interior = np.all((coords > 0) & (coords < ne), axis=1)
    if jitter:
        coords[interior] += rng.uniform(-jitter, jitter, size=(int(interior.sum()), 3))
    coords *= h
    ci, cj, ck = (a.ravel() for a in np.meshgrid(np.arange(ne), np.arange(ne), np.arange(ne), indexing="ij"))

    def nid(i, j, k):
        return (i * (ne + 1) + j) * (ne + 1) + k

    tets = []
    for perm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        cur = [ci.copy(), cj.copy(), ck.copy()]
        vs = [nid(*cur)]
        for ax in perm:
            cur[ax] = cur[ax] + 1
            vs.append(nid(*cur))
        tets.append(np.stack(vs, axis=1))
    tets = np.stack(tets, axis=1).reshape(-1, 4)
    p = coords[tets]
    det = np.linalg.det(p[:, 1:] - p[:, :1])
    neg = det < 0
    tets[neg, 1], tets[neg, 2] = tets[neg, 2].copy(), tets[neg, 1].copy()
    return coords, tets


def extract_defect_dofs(elements, gid):
    """final_assembly.py:27-57."""
    mask = elements[:, -1] == 1
    if not mask.any():
        return np.zeros(0, dtype=np.int32)
    nodes = np.unique(elements[mask, :-1].ravel())
    return np.unique(gid[nodes]).astype(np.int32)
