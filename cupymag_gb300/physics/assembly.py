"""FEM operator assembly on the host (setup; runs once per mesh).

Element integrals follow the reference assemblers
(cupymag/physics/assemble_demag.py:95-184, assemble_Gauss_Seidel.py:88-161,
assemble_elasticity.py:194-348): gradients J^{-1} dN/dxi with the shape
module's Jacobian convention, signed detJ, Gauss tables of mesh/shapes.py,
all-zero element matrices when |detJ| < 1e-14 at a point.  They are
vectorised over elements instead of JIT loops.

Two global assemblies produce the same CSR matrices:
* ``assemble_coo``: general meshes (tets, small hex grids) -- element COO in
  the reference's ordering, summed by SciPy's COO->CSR (final_assembly.py:160-205);
* ``structured_hex`` (physics/structured_hex.py): periodic unit-cell hex grids,
  built straight into CSR from one element matrix and the 27-point periodic
  stencil, on the GPU, without the Ne*(3*8)*(6*8) host COO arrays.
Both then apply the anchor rows/columns and the defect enforcement of
final_assembly.py:59-158.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from ..mesh import shapes


def _tables(nen):
    return shapes.hex_assembly_tables() if nen == 8 else shapes.tet_assembly_tables()


def element_gradients(xe):
    """xe: (Ne, nen, 3) corner coordinates -> grads (Ne,ngp,nen,3), N (ngp,nen), wdet (Ne,ngp), zero (Ne,)."""
    Ne, nen, _ = xe.shape
    dN, N, w = _tables(nen)
    ngp = len(w)
    grads = np.empty((Ne, ngp, nen, 3))
    wdet = np.empty((Ne, ngp))
    zero = np.zeros(Ne, dtype=bool)
    eye = np.eye(3)
    for g in range(ngp):
        if nen == 8:
            J = np.einsum("eak,aj->ekj", xe, dN[g])      # J[k, j] = d x_k / d xi_j   (ShapeHex.py:237-249)
        else:
            J = xe[:, 1:, :] - xe[:, :1, :]              # rows are edge vectors      (ShapeTet.py:196-200)
        det = np.linalg.det(J)
        bad = np.abs(det) < 1e-14
        zero |= bad
        if bad.any():
            J = J.copy()
            J[bad] = eye
        grads[:, g] = np.einsum("eij,aj->eai", np.linalg.inv(J), dN[g])
        wdet[:, g] = det * w[g]
    return grads, N, wdet, zero


def scalar_element_matrices(xe):
    """K_e = (grad N_a, grad N_b), M_e = (N_a, N_b), F_e,i = (N_a, dN_b/dx_i)."""
    grads, N, wdet, zero = element_gradients(xe)
    K = np.einsum("egai,egbi,eg->eab", grads, grads, wdet)
    M = np.einsum("ga,gb,eg->eab", N, N, wdet)
    F = [np.einsum("ga,egb,eg->eab", N, grads[..., i], wdet) for i in range(3)]
    for X in [K, M, *F]:
        X[zero] = 0.0
    return K, M, F


def stiffness_voigt(c11, c12, c44, Mrot=None):
    """Cubic 6x6 Voigt stiffness, rotated as M C M^T for the [111] frame (assemble_elasticity.py:175-192)."""
    C = np.zeros((6, 6))
    C[:3, :3] = c12
    np.fill_diagonal(C[:3, :3], c11)
    C[3, 3] = C[4, 4] = C[5, 5] = c44
    if Mrot is not None:
        C = Mrot @ C @ Mrot.T
    return C


def elastic_element_matrices(xe, C):
    """K_el (Ne, 3nen, 3nen) = sum B^T C B |J| w;  F_el (Ne, 3nen, 6nen) = sum B^T C S |J| w."""
    grads, N, wdet, zero = element_gradients(xe)
    Ne, ngp, nen, _ = grads.shape
    K = np.zeros((Ne, 3 * nen, 3 * nen))
    F = np.zeros((Ne, 3 * nen, 6 * nen))
    # strain-displacement rows [xx, yy, zz, xy, yz, xz] (assemble_elasticity.py:241-252)
    pairs = ((0, 0, 0), (1, 1, 1), (2, 2, 2), (3, 0, 1), (3, 1, 0), (4, 1, 2), (4, 2, 1), (5, 0, 2), (5, 2, 0))
    for g in range(ngp):
        B = np.zeros((Ne, 6, nen, 3))
        for row, comp, dirn in pairs:
            B[:, row, :, comp] = grads[:, g, :, dirn]
        B = B.reshape(Ne, 6, 3 * nen)
        BtC = np.einsum("eki,kj->eij", B, C)
        K += np.einsum("eik,ekj->eij", BtC, B) * wdet[:, g, None, None]
        F += (BtC[:, :, None, :] * N[g][None, None, :, None]).reshape(Ne, 3 * nen, 6 * nen) * wdet[:, g, None, None]
    K[zero] = 0.0
    F[zero] = 0.0
    return K, F


# ------------------------------------------------------------------ CSR helpers
def to_csr(rows, cols, vals, shape):
    return sp.coo_matrix((vals, (rows, cols)), shape=shape).tocsr()


def zero_rows_cols(A: sp.csr_matrix, anchors, cols_too=True, diag_one=True):
    """Zero row (and column) entries of the anchor DOFs, set the anchor diagonal to 1.

    The entries stay stored as explicit zeros, as the reference's COO anchoring
    does (assemble_demag.py:307-341, assemble_elasticity.py:461-527).
    """
    A = A.copy()
    rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    an = np.asarray(anchors)
    hit = np.isin(rows, an)
    if cols_too:
        hit |= np.isin(A.indices, an)
    A.data[hit] = 0.0
    if diag_one:
        for a in anchors:
            s, e = A.indptr[a], A.indptr[a + 1]
            k = s + np.searchsorted(A.indices[s:e], a)
            if k < e and A.indices[k] == a:
                A.data[k] = 1.0
            else:
                raise ValueError("anchor diagonal missing from the pattern")
    return A


def enforce_defect_A(A: sp.csr_matrix, defect):
    """final_assembly.py:59-111: drop defect rows/columns, unit diagonal on defect DOFs."""
    if defect is None or len(defect) == 0:
        return A
    isd = np.zeros(A.shape[0], dtype=bool)
    isd[defect] = True
    rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    keep = ~(isd[rows] | isd[A.indices])
    cnt = np.bincount(rows[keep], minlength=A.shape[0])
    cnt[isd] = 1
    indptr = np.zeros(A.shape[0] + 1, dtype=np.int64)
    np.cumsum(cnt, out=indptr[1:])
    indices = np.empty(indptr[-1], dtype=np.int32)
    data = np.empty(indptr[-1])
    kept_rows = rows[keep]
    kc = np.bincount(kept_rows, minlength=A.shape[0])
    kcum = np.concatenate([[0], np.cumsum(kc)[:-1]])
    pos = indptr[kept_rows] + (np.arange(kept_rows.size) - kcum[kept_rows])
    indices[pos] = A.indices[keep]
    data[pos] = A.data[keep]
    indices[indptr[defect]] = defect
    data[indptr[defect]] = 1.0
    return sp.csr_matrix((data, indices, indptr), shape=A.shape)


def enforce_defect_F(F: sp.csr_matrix, defect):
    """final_assembly.py:114-158: drop the rows of defect DOFs."""
    if defect is None or len(defect) == 0:
        return F
    isd = np.zeros(F.shape[0], dtype=bool)
    isd[defect] = True
    cnt = np.diff(F.indptr).copy()
    rows = np.repeat(np.arange(F.shape[0]), cnt)
    keep = ~isd[rows]
    cnt[isd] = 0
    indptr = np.zeros(F.shape[0] + 1, dtype=np.int64)
    np.cumsum(cnt, out=indptr[1:])
    return sp.csr_matrix((F.data[keep], F.indices[keep], indptr), shape=F.shape)


# ------------------------------------------------------------------ general COO path
def assemble_coo(coords, elements, gid, n, defect, alpha1, alpha2, ME=False, C=None):
    """All operators of SimulationOperators (assemble_simulation_operators.py:42-107) as SciPy CSR."""
    nen = elements.shape[1] - 1
    xe = coords[elements[:, :nen]]
    d = gid[elements[:, :nen]].astype(np.int64)
    Ne = len(d)
    K, M, F = scalar_element_matrices(xe)
    rows = np.repeat(d, nen, axis=1).ravel()
    cols = np.tile(d, (1, nen)).ravel()
    ops = {}
    Kc = to_csr(rows, cols, K.ravel(), (n, n))
    ops["A_demag"] = zero_rows_cols(Kc, [0])
    for nm, Fi in zip(("Fx", "Fy", "Fz"), F):
        ops[nm] = to_csr(rows, cols, Fi.ravel(), (n, n))
    ops["A1"] = enforce_defect_A(to_csr(rows, cols, K.ravel() * alpha1 + M.ravel(), (n, n)), defect)
    ops["A2"] = enforce_defect_A(to_csr(rows, cols, K.ravel() * alpha2 + M.ravel(), (n, n)), defect)
    ops["F1"] = enforce_defect_F(to_csr(rows, cols, M.ravel(), (n, n)), defect)
    if ME:
        Kel, Fel = elastic_element_matrices(xe, C)
        r3 = (d[:, :, None] + n * np.arange(3)[None, None, :]).reshape(Ne, 3 * nen)
        c6 = (6 * d[:, :, None] + np.arange(6)[None, None, :]).reshape(Ne, 6 * nen)
        A = to_csr(np.repeat(r3, 3 * nen, axis=1).ravel(), np.tile(r3, (1, 3 * nen)).ravel(), Kel.ravel(),
                   (3 * n, 3 * n))
        ops["A_el"] = zero_rows_cols(A, [0, n, 2 * n])
        Fm = to_csr(np.repeat(r3, 6 * nen, axis=1).ravel(), np.tile(c6, (1, 3 * nen)).ravel(), Fel.ravel(),
                    (3 * n, 6 * n))
        ops["F_el"] = zero_rows_cols(Fm, [0, n, 2 * n], cols_too=False, diag_one=False)
    return ops
