"""FEM assembly (oracle restatement), vectorised over elements.

Element matrices follow the reference's per-element loops:
* scalar K_e = (grad N_a, grad N_b), M_e = (N_a, N_b),
  F_e,i = (N_a, dN_b/dx_i)  (assemble_demag.py:95-184,
  assemble_Gauss_Seidel.py:88-161);
* elasticity K_e = B^T C B, F_e = B^T C S  (assemble_elasticity.py:194-348),
  with C rotated as M C M^T when rot111 (assemble_elasticity.py:61-98,190-192);
* gradients are J^{-1} dN/dxi with J from element_jacobian of the shape module
  (hex: ShapeHex.py:216-251; tet: ShapeTet.py:175-202); the signed detJ weights
  the integrand; an element with |detJ| < 1e-14 at any point contributes an
  all-zero matrix (assemble_demag.py:116-117).
Global COO ordering per element: a, b (scalar); a, da, b, db (A_el);
a, da, b, vb (F_el) (assemble_elasticity.py:389-398,444-454).
Anchors: A_demag zeroes row/col 0 and appends (0,0,1)
(assemble_demag.py:307-341); A_el does so for DOFs 0, n, 2n; F_el zeroes rows
0, n, 2n (assemble_elasticity.py:461-527).  COO -> CSR by SciPy, and defect
enforcement of final_assembly.py:59-205.
"""
import numpy as np
import scipy.sparse as sp

from . import shapes


def _tables(nen):
    if nen == 8:
        dN, N = shapes.hex_tables()
        _, w = shapes.hex_gauss()
    else:
        dN, N = shapes.tet_tables()
        _, w = shapes.tet_gauss()
    return dN, N, w


def _jacobians(xe, igp_dN, nen):
    """J per element at one Gauss point (Ne,3,3), reference conventions."""
    if nen == 8:
        # J[k, j] = sum_i x_i[k] dN[i, j]   (ShapeHex.py:240-249)
        return np.einsum("eik,ij->ekj", xe, igp_dN)
    # J[:, k] = coord_k[1:] - coord_k[0]  (ShapeTet.py:196-200)
    return xe[:, 1:, :] - xe[:, :1, :]


def element_data(coords, elements):
    """Per-element, per-Gauss-point gradients, N and signed detJ*w.

    Returns grads (Ne, ngp, nen, 3), Nt (ngp, nen), dw (Ne, ngp), zero (Ne,)
    where zero flags elements that have |detJ| < 1e-14 at some point.
    """
    nen = elements.shape[1] - 1
    dN, N, w = _tables(nen)
    xe = coords[elements[:, :nen]]  # (Ne, nen, 3)
    ngp = len(w)
    Ne = elements.shape[0]
    grads = np.empty((Ne, ngp, nen, 3))
    dw = np.empty((Ne, ngp))
    zero = np.zeros(Ne, dtype=bool)
    for g in range(ngp):
        J = _jacobians(xe, dN[g], nen)
        det = np.linalg.det(J)
        bad = np.abs(det) < 1e-14
        zero |= bad
        Jg = J.copy()
        Jg[bad] = np.eye(3)
        Jinv = np.linalg.inv(Jg)
        grads[:, g] = np.einsum("eij,aj->eai", Jinv, dN[g])
        dw[:, g] = det * w[g]
    return grads, N, dw, zero


def scalar_element_matrices(coords, elements):
    """K_e, M_e, Fx_e, Fy_e, Fz_e, each (Ne, nen, nen)."""
    grads, N, dw, zero = element_data(coords, elements)
    K = np.einsum("egai,egbi,eg->eab", grads, grads, dw)
    M = np.einsum("ga,gb,eg->eab", N, N, dw)
    F = [np.einsum("ga,egb,eg->eab", N, grads[..., i], dw) for i in range(3)]
    for A in [K, M] + F:
        A[zero] = 0.0
    return K, M, F[0], F[1], F[2]


def voigt_C(c11, c12, c44, rot111, Mrot=None):
    C = np.zeros((6, 6))
    C[:3, :3] = c12
    C[0, 0] = C[1, 1] = C[2, 2] = c11
    C[3, 3] = C[4, 4] = C[5, 5] = c44
    if rot111:
        C = Mrot @ C @ Mrot.T
    return C


def _B(grads_g):
    """B (Ne, 6, 3nen) from gradients at one Gauss point (assemble_elasticity.py:228-252)."""
    Ne, nen, _ = grads_g.shape
    B = np.zeros((Ne, 6, 3 * nen))
    gx, gy, gz = grads_g[..., 0], grads_g[..., 1], grads_g[..., 2]
    B[:, 0, 0::3] = gx
    B[:, 1, 1::3] = gy
    B[:, 2, 2::3] = gz
    B[:, 3, 0::3] = gy
    B[:, 3, 1::3] = gx
    B[:, 4, 1::3] = gz
    B[:, 4, 2::3] = gy
    B[:, 5, 0::3] = gz
    B[:, 5, 2::3] = gx
    return B


def elastic_element_matrices(coords, elements, C):
    """Kel_e (Ne, 3nen, 3nen) and Fel_e (Ne, 3nen, 6nen)."""
    grads, N, dw, zero = element_data(coords, elements)
    Ne, ngp, nen, _ = grads.shape
    K = np.zeros((Ne, 3 * nen, 3 * nen))
    F = np.zeros((Ne, 3 * nen, 6 * nen))
    for g in range(ngp):
        B = _B(grads[:, g])
        BtC = np.einsum("eki,kj->eij", B, C)
        K += np.einsum("eik,ekj->eij", BtC, B) * dw[:, g, None, None]
        # S[v, 6a+v] = N_a -> F[i, 6a+v] = BtC[i, v] N_a
        Fg = np.einsum("eiv,a->eiav", BtC, N[g]).reshape(Ne, 3 * nen, 6 * nen)
        F += Fg * dw[:, g, None, None]
    K[zero] = 0.0
    F[zero] = 0.0
    return K, F


def scalar_coo(elements, gid, Ke):
    nen = elements.shape[1] - 1
    d = gid[elements[:, :nen]]
    rows = np.repeat(d, nen, axis=1).ravel()
    cols = np.tile(d, (1, nen)).ravel()
    return rows.astype(np.int32), cols.astype(np.int32), Ke.reshape(-1).copy()


def elastic_coo_A(elements, gid, Ke, n):
    nen = elements.shape[1] - 1
    d = gid[elements[:, :nen]].astype(np.int64)
    Ne = d.shape[0]
    ra = (d[:, :, None] + np.arange(3)[None, None, :] * n).reshape(Ne, 3 * nen)  # index 3a+da
    rows = np.repeat(ra, 3 * nen, axis=1).ravel()
    cols = np.tile(ra, (1, 3 * nen)).ravel()
    return rows.astype(np.int32), cols.astype(np.int32), Ke.reshape(-1).copy()


def elastic_coo_F(elements, gid, Fe, n):
    nen = elements.shape[1] - 1
    d = gid[elements[:, :nen]].astype(np.int64)
    Ne = d.shape[0]
    ra = (d[:, :, None] + np.arange(3)[None, None, :] * n).reshape(Ne, 3 * nen)
    cb = (d[:, :, None] * 6 + np.arange(6)[None, None, :]).reshape(Ne, 6 * nen)
    rows = np.repeat(ra, 6 * nen, axis=1).ravel()
    cols = np.tile(cb, (1, 3 * nen)).ravel()
    return rows.astype(np.int32), cols.astype(np.int32), Fe.reshape(-1).copy()


def anchor_A(rows, cols, vals, anchors):
    vals = vals.copy()
    for a in anchors:
        vals[(rows == a) | (cols == a)] = 0.0
    rows = np.concatenate([rows, np.asarray(anchors, dtype=rows.dtype)])
    cols = np.concatenate([cols, np.asarray(anchors, dtype=cols.dtype)])
    vals = np.concatenate([vals, np.ones(len(anchors))])
    return rows, cols, vals


def anchor_F(rows, cols, vals, anchors):
    vals = vals.copy()
    for a in anchors:
        vals[rows == a] = 0.0
    return rows, cols, vals


def to_csr(rows, cols, vals, shape):
    return sp.coo_matrix((vals, (rows, cols)), shape=shape).tocsr()


def enforce_defect_A(A, defect):
    """final_assembly.py:59-111: drop rows/cols of defect DOFs, add identity."""
    if defect is None or len(defect) == 0:
        return A
    C = A.tocoo()
    dmask = np.zeros(A.shape[0], dtype=bool)
    dmask[defect] = True
    keep = ~(dmask[C.row] | dmask[C.col])
    r = np.concatenate([C.row[keep], defect])
    c = np.concatenate([C.col[keep], defect])
    v = np.concatenate([C.data[keep], np.ones(len(defect))])
    return sp.coo_matrix((v, (r, c)), shape=A.shape).tocsr()


def enforce_defect_F(F, defect):
    """final_assembly.py:114-158: drop the rows of defect DOFs."""
    if defect is None or len(defect) == 0:
        return F
    C = F.tocoo()
    dmask = np.zeros(F.shape[0], dtype=bool)
    dmask[defect] = True
    keep = ~dmask[C.row]
    return sp.coo_matrix((C.data[keep], (C.row[keep], C.col[keep])), shape=F.shape).tocsr()


def build_operators(coords, elements, gid, n, defect, alpha1, alpha2, ME=False, C=None):
    """All matrices of SimulationOperators (assemble_simulation_operators.py:42-107)."""
    K, M, Fx, Fy, Fz = scalar_element_matrices(coords, elements)
    r, c, vK = scalar_coo(elements, gid, K)
    _, _, vM = scalar_coo(elements, gid, M)
    ops = {}
    ra, ca, va = anchor_A(r, c, vK.copy(), [0])
    ops["A_demag"] = to_csr(ra, ca, va, (n, n))
    for name, Fe in (("Fx", Fx), ("Fy", Fy), ("Fz", Fz)):
        _, _, v = scalar_coo(elements, gid, Fe)
        ops[name] = to_csr(r, c, v, (n, n))
    ops["A1"] = enforce_defect_A(to_csr(r, c, vK * alpha1 + vM, (n, n)), defect)
    ops["A2"] = enforce_defect_A(to_csr(r, c, vK * alpha2 + vM, (n, n)), defect)
    ops["F1"] = enforce_defect_F(to_csr(r, c, vM, (n, n)), defect)
    if ME:
        Ke, Fe = elastic_element_matrices(coords, elements, C)
        rA, cA, vA = elastic_coo_A(elements, gid, Ke, n)
        rA, cA, vA = anchor_A(rA, cA, vA, [0, n, 2 * n])
        ops["A_el"] = to_csr(rA, cA, vA, (3 * n, 3 * n))
        rF, cF, vF = elastic_coo_F(elements, gid, Fe, n)
        rF, cF, vF = anchor_F(rF, cF, vF, [0, n, 2 * n])
        ops["F_el"] = to_csr(rF, cF, vF, (3 * n, 6 * n))
    return ops
