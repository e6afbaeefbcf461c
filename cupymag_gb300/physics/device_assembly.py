"""FEM operator assembly on the GPU for unstructured meshes (setup; runs once per mesh).

The same element integrals as ``physics/assembly.py`` (cupymag/physics/
assemble_demag.py:95-184, assemble_Gauss_Seidel.py:88-161,
assemble_elasticity.py:194-348: gradients J^{-1} dN/dxi, signed detJ, the
shape module's Gauss tables, all-zero element matrices when |detJ| < 1e-14),
evaluated with torch on the device in blocks of elements; the COO triplets
stay on the device and are summed into CSR by a stable sort on (row, col)
followed by ``cpm_coo_segment_sum`` (duplicates added in element order, so
the result is deterministic).  Anchors and defects use the device CSR
helpers of ``physics/structured_hex.py``.  This replaces the host COO path
for meshes whose triplets do not fit comfortably in host memory (a 96^3
Kuhn-tet mesh has 1.5e9 F_el triplets).
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _native as N
from ..mesh import shapes
from . import structured_hex as SH

_BLOCK = 1 << 19  # elements per block


def _tables(nen, dev):
    dN, Nt, w = shapes.hex_assembly_tables() if nen == 8 else shapes.tet_assembly_tables()
    f = lambda a: torch.as_tensor(np.asarray(a), dtype=torch.float64, device=dev)  # noqa: E731
    return f(dN), f(Nt), [float(v) for v in np.asarray(w)]


def element_gradients(xe):
    """Torch form of physics.assembly.element_gradients: xe (Ne, nen, 3) on the device."""
    Ne, nen, _ = xe.shape
    dN, Nt, w = _tables(nen, xe.device)
    ngp = len(w)
    grads = torch.empty((Ne, ngp, nen, 3), dtype=torch.float64, device=xe.device)
    wdet = torch.empty((Ne, ngp), dtype=torch.float64, device=xe.device)
    zero = torch.zeros(Ne, dtype=torch.bool, device=xe.device)
    eye = torch.eye(3, dtype=torch.float64, device=xe.device)
    for g in range(ngp):
        if nen == 8:
            J = torch.einsum("eak,aj->ekj", xe, dN[g])
        else:
            J = xe[:, 1:, :] - xe[:, :1, :]
        det = torch.linalg.det(J)
        bad = det.abs() < 1e-14
        zero |= bad
        if bool(bad.any()):
            J = J.clone()
            J[bad] = eye
        grads[:, g] = torch.einsum("eij,aj->eai", torch.linalg.inv(J), dN[g])
        wdet[:, g] = det * w[g]
    return grads, Nt, wdet, zero


def scalar_element_matrices(xe):
    grads, Nt, wdet, zero = element_gradients(xe)
    K = torch.einsum("egai,egbi,eg->eab", grads, grads, wdet)
    M = torch.einsum("ga,gb,eg->eab", Nt, Nt, wdet)
    F = [torch.einsum("ga,egb,eg->eab", Nt, grads[..., i], wdet) for i in range(3)]
    for X in [K, M, *F]:
        X[zero] = 0.0
    return K, M, F


def elastic_element_matrices(xe, C):
    grads, Nt, wdet, zero = element_gradients(xe)
    Ne, ngp, nen, _ = grads.shape
    Ct = torch.as_tensor(C, dtype=torch.float64, device=xe.device)
    K = torch.zeros((Ne, 3 * nen, 3 * nen), dtype=torch.float64, device=xe.device)
    F = torch.zeros((Ne, 3 * nen, 6 * nen), dtype=torch.float64, device=xe.device)
    pairs = ((0, 0, 0), (1, 1, 1), (2, 2, 2), (3, 0, 1), (3, 1, 0), (4, 1, 2), (4, 2, 1), (5, 0, 2), (5, 2, 0))
    for g in range(ngp):
        B = torch.zeros((Ne, 6, nen, 3), dtype=torch.float64, device=xe.device)
        for row, comp, dirn in pairs:
            B[:, row, :, comp] = grads[:, g, :, dirn]
        B = B.reshape(Ne, 6, 3 * nen)
        BtC = torch.einsum("eki,kj->eij", B, Ct)
        K += torch.einsum("eik,ekj->eij", BtC, B) * wdet[:, g, None, None]
        F += (BtC[:, :, None, :] * Nt[g][None, None, :, None]).reshape(Ne, 3 * nen, 6 * nen) * wdet[:, g, None, None]
    K[zero] = 0.0
    F[zero] = 0.0
    return K, F


class _COO:
    """Device COO accumulator: keys row * ncols + col and values, in element order."""

    def __init__(self, shape):
        self.shape = shape
        self.keys, self.vals = [], []

    def add(self, rows, cols, vals):
        self.keys.append((rows * self.shape[1] + cols).reshape(-1))
        self.vals.append(vals.reshape(-1))

    def csr(self):
        keys = torch.cat(self.keys)
        vals = torch.cat(self.vals)
        self.keys, self.vals = [], []
        keys, perm = torch.sort(keys, stable=True)
        vals = vals[perm]
        del perm
        uk, counts = torch.unique_consecutive(keys, return_counts=True)
        del keys
        start = torch.zeros(uk.numel() + 1, dtype=torch.int64, device=uk.device)
        torch.cumsum(counts, 0, out=start[1:])
        data = torch.empty(uk.numel(), dtype=torch.float64, device=uk.device)
        N.check(N.lib().cpm_coo_segment_sum(vals.data_ptr(), start.data_ptr(), uk.numel(), data.data_ptr(),
                                            N.stream_ptr()), "cpm_coo_segment_sum")
        del vals, start
        nrows, ncols = self.shape
        rows = torch.div(uk, ncols, rounding_mode="floor")
        cols = (uk - rows * ncols).to(torch.int32)
        indptr = torch.zeros(nrows + 1, dtype=torch.int64, device=uk.device)
        torch.cumsum(torch.bincount(rows, minlength=nrows), 0, out=indptr[1:])
        return indptr, cols, data


def assemble_device(coords, elements, gid, n, defect, alpha1, alpha2, ME=False, C=None, device=None):
    """All operators of SimulationOperators as device CSR triples (indptr, indices, data).

    Same results as physics.assembly.assemble_coo up to the summation order of
    duplicate entries."""
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    nen = elements.shape[1] - 1
    Ne = len(elements)
    coords_t = torch.as_tensor(np.asarray(coords, dtype=np.float64), device=dev)
    elem_t = torch.as_tensor(np.asarray(elements[:, :nen], dtype=np.int64), device=dev)
    gid_t = torch.as_tensor(np.asarray(gid, dtype=np.int64), device=dev)
    scal = {k: _COO((n, n)) for k in ("K", "M", "Fx", "Fy", "Fz")}
    coo_el = {"A_el": _COO((3 * n, 3 * n)), "F_el": _COO((3 * n, 6 * n))} if ME else {}

    def blocks():
        for e0 in range(0, Ne, _BLOCK):
            el = elem_t[e0:e0 + _BLOCK]
            yield coords_t[el], gid_t[el]

    # scalar operators: every block's K, M, F_x,y,z entries
    for xe, d in blocks():
        K, M, F = scalar_element_matrices(xe)
        rows = d[:, :, None].expand(-1, nen, nen)
        cols = d[:, None, :].expand(-1, nen, nen)
        for key, X in zip(("K", "M", "Fx", "Fy", "Fz"), (K, M, *F)):
            scal[key].add(rows, cols, X)
    ops = {}
    # A1 / A2 = K alpha + M need the summed K and M with the same pattern: sum them separately
    Kc = scal["K"].csr()
    Mc = scal["M"].csr()
    if not (torch.equal(Kc[0], Mc[0]) and torch.equal(Kc[1], Mc[1])):
        raise RuntimeError("K and M patterns differ")
    ops["A_demag"] = SH.anchor(*Kc, (0,))
    for nm in ("Fx", "Fy", "Fz"):
        ops[nm] = scal[nm].csr()
    ip, ix = Kc[0], Kc[1]
    for nm, a in (("A1", alpha1), ("A2", alpha2)):
        ops[nm] = SH.drop_defect(ip, ix, Kc[2] * a + Mc[2], defect, cols_too=True, unit_diag=True)
    ops["F1"] = SH.drop_defect(ip, ix, Mc[2].clone(), defect, cols_too=False, unit_diag=False)
    del Kc, Mc
    if ME:
        ar3 = torch.arange(3, device=dev)
        ar6 = torch.arange(6, device=dev)
        for key in ("A_el", "F_el"):
            for xe, d in blocks():
                Kel, Fel = elastic_element_matrices(xe, C)
                r3 = (d[:, :, None] + n * ar3[None, None, :]).reshape(len(d), 3 * nen)
                if key == "A_el":
                    coo_el[key].add(r3[:, :, None].expand(-1, -1, 3 * nen), r3[:, None, :].expand(-1, 3 * nen, -1),
                                    Kel)
                else:
                    c6 = (6 * d[:, :, None] + ar6[None, None, :]).reshape(len(d), 6 * nen)
                    coo_el[key].add(r3[:, :, None].expand(-1, -1, 6 * nen), c6[:, None, :].expand(-1, 3 * nen, -1),
                                    Fel)
                del Kel, Fel
            t = coo_el[key].csr()
            if key == "A_el":
                ops[key] = SH.anchor(*t, (0, n, 2 * n))
            else:
                ops[key] = SH.anchor(*t, (0, n, 2 * n), cols_too=False, diag_one=False)
    return ops
