"""Meshes, periodic DOF maps and defect DOFs (oracle restatement).

* HexGrid.std_fem_mesh (cupymag/mesh/gridHex.py:68-142): nodes i-major with k
  fastest, node_id = i(Ny+1)(Nz+1) + j(Nz+1) + k; elements in i, j, k order
  with the corner order of gridHex.py:119-126; an element is a defect when its
  centre lies in [c - Nd/2, c + Nd/2) on every axis.
* build_periodic_node_map (gridHex.py:179-213, gridTet.py:180-225): wrap the
  coordinate that equals the domain maximum onto the minimum, round to 12
  decimals, number keys in first-appearance order.  Restated literally (a dict
  loop) so that it can pin the closed forms the product uses.
* extract_defect_dofs (cupymag/utils/final_assembly.py:27-57).
* TetraGrid defect flags by element centroid (gridTet.py:154-178) and the
  defect shapes of cupymag/utils/defect_shapes.py:73-134.
"""
import numpy as np


def hex_mesh(Nx, Ny, Nz, Ndx, Ndy, Ndz, defect_center=None):
    x = np.linspace(0, Nx, Nx + 1)
    y = np.linspace(0, Ny, Ny + 1)
    z = np.linspace(0, Nz, Nz + 1)
    i3, j3, k3 = np.meshgrid(np.arange(Nx + 1), np.arange(Ny + 1), np.arange(Nz + 1), indexing="ij")
    coords = np.stack((x[i3.ravel()], y[j3.ravel()], z[k3.ravel()]), axis=1)
    if defect_center is None:
        cx, cy, cz = Nx / 2.0, Ny / 2.0, Nz / 2.0
    else:
        cx, cy, cz = defect_center
    lo = (cx - Ndx / 2.0, cy - Ndy / 2.0, cz - Ndz / 2.0)
    hi = (cx + Ndx / 2.0, cy + Ndy / 2.0, cz + Ndz / 2.0)

    def node_id(ii, jj, kk):
        return ii * (Ny + 1) * (Nz + 1) + jj * (Nz + 1) + kk

    ei, ej, ek = np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing="ij")
    ei, ej, ek = ei.ravel(), ej.ravel(), ek.ravel()
    el = np.zeros((Nx * Ny * Nz, 9), dtype=np.int32)
    el[:, 0] = node_id(ei, ej, ek)
    el[:, 1] = node_id(ei + 1, ej, ek)
    el[:, 2] = node_id(ei + 1, ej + 1, ek)
    el[:, 3] = node_id(ei, ej + 1, ek)
    el[:, 4] = node_id(ei, ej, ek + 1)
    el[:, 5] = node_id(ei + 1, ej, ek + 1)
    el[:, 6] = node_id(ei + 1, ej + 1, ek + 1)
    el[:, 7] = node_id(ei, ej + 1, ek + 1)
    xc, yc, zc = ei + 0.5, ej + 0.5, ek + 0.5
    dfl = ((xc >= lo[0]) & (xc < hi[0]) & (yc >= lo[1]) & (yc < hi[1]) & (zc >= lo[2]) & (zc < hi[2]))
    el[:, 8] = dfl.astype(np.int32)
    return coords, el


def periodic_node_map(coords, lo, hi, tol=1e-12):
    canon = {}
    gid = np.zeros(coords.shape[0], dtype=np.int32)
    nxt = 0
    for n in range(coords.shape[0]):
        key = []
        for d in range(3):
            v = coords[n, d]
            if abs(v - hi[d]) < tol:
                v = float(lo[d])
            key.append(round(float(v), 12))
        key = tuple(key)
        if key not in canon:
            canon[key] = nxt
            nxt += 1
        gid[n] = canon[key]
    return gid


def hex_periodic_map(Nx, Ny, Nz, coords):
    return periodic_node_map(coords, (0.0, 0.0, 0.0), (float(Nx), float(Ny), float(Nz)))


def tet_periodic_map(coords):
    return periodic_node_map(coords, coords.min(axis=0), coords.max(axis=0))


def extract_defect_dofs(elements, gid):
    mask = elements[:, -1] == 1
    if not mask.any():
        return np.asarray([], dtype=np.int32)
    nodes = np.unique(elements[mask, :-1].ravel())
    return np.unique(gid[nodes]).astype(np.int32)


def defect_indicator(shape, params, rotation=None):
    if shape == "Sphere":
        R2 = float(params) ** 2 if np.ndim(params) == 0 else float(params[0]) ** 2
        return lambda rel: np.sum(rel ** 2, axis=1) < R2
    if shape == "Ellipsoid":
        a, b, c = params
        inv2 = np.array([1.0 / a ** 2, 1.0 / b ** 2, 1.0 / c ** 2])
        return lambda rel: np.sum(rel ** 2 * inv2[None, :], axis=1) < 1.0
    if shape == "RotatedEllipsoid":
        a, b, c = params
        R = np.asarray(rotation, dtype=float)
        Q = R @ np.diag([1.0 / a ** 2, 1.0 / b ** 2, 1.0 / c ** 2]) @ R.T
        return lambda rel: np.sum((rel @ Q) * rel, axis=1) < 1.0
    raise NotImplementedError(shape)


def tet_elements(coords, tets, indicator, defect_center=None):
    if defect_center is None:
        defect_center = (coords.min(axis=0) + coords.max(axis=0)) / 2
    el = np.zeros((tets.shape[0], 5), dtype=np.int32)
    el[:, :4] = tets
    centers = coords[el[:, :4]].mean(axis=1)
    el[:, 4] = indicator(centers - np.asarray(defect_center)).astype(np.int32)
    return el
