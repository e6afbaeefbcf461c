"""Direct CSR assembly for periodic grids of identical unit hex cells.

Every cell of HexGrid is the same unit cube, so each global operator is a
27-point periodic stencil: the coefficient between DOF p and DOF p + d
(d in {-1,0,1}^3, wrapped) is the sum over the eight cells that contain both
of one element-matrix entry K_e[a, b] with offset(b) - offset(a) = d.  The CSR
rows are written directly from that stencil with columns in ascending order,
which for each axis is [0,+1,-1] at index 0, [+1,-1,0] at index N-1 and
[-1,0,+1] elsewhere.  The result has the same pattern as the reference's
COO -> CSR assembly (assemble_demag.py:186-233, assemble_Gauss_Seidel.py:163-214,
assemble_elasticity.py:350-459); values agree to rounding (the reference sums
per-element copies of the same element matrix).

The index arithmetic runs as torch tensor ops on the target device, so the
128^3 elastic operators (0.5 G and 1 G non-zeros) are built in GPU memory in
well under a second instead of through tens of GB of host COO arrays.
Requires Nx, Ny, Nz >= 3 (smaller grids alias neighbours; use the COO path).
"""
from __future__ import annotations

import numpy as np
import torch

from ..mesh.shapes import HEX_OFFSETS


def stencil_from_element(Ke, rdim=1, cdim=1):
    """(rdim, cdim, 3, 3, 3) stencil from a (8*rdim, 8*cdim) element matrix (node-major blocks)."""
    S = np.zeros((rdim, cdim, 3, 3, 3))
    for a in range(8):
        for b in range(8):
            d = HEX_OFFSETS[b] - HEX_OFFSETS[a] + 1
            S[:, :, d[0], d[1], d[2]] += Ke[a * rdim:(a + 1) * rdim, b * cdim:(b + 1) * cdim]
    return S


def _axis_order(N, device):
    o = torch.empty((N, 3), dtype=torch.int64, device=device)
    o[:] = torch.tensor([-1, 0, 1], device=device)
    o[0] = torch.tensor([0, 1, -1], device=device)
    o[N - 1] = torch.tensor([1, -1, 0], device=device)
    return o


def _pattern(Nx, Ny, Nz, device):
    """Neighbour columns (n, 27) in ascending order and the stencil offset of each (n, 27) as 0..26."""
    ox, oy, oz = _axis_order(Nx, device), _axis_order(Ny, device), _axis_order(Nz, device)
    ix = torch.arange(Nx, device=device)[:, None]
    iy = torch.arange(Ny, device=device)[:, None]
    iz = torch.arange(Nz, device=device)[:, None]
    cx = ((ix + ox) % Nx) * (Ny * Nz)          # (Nx, 3)
    cy = ((iy + oy) % Ny) * Nz                 # (Ny, 3)
    cz = (iz + oz) % Nz                        # (Nz, 3)
    cols = (cx[:, None, None, :, None, None] + cy[None, :, None, None, :, None]
            + cz[None, None, :, None, None, :]).reshape(-1, 27)
    sx, sy, sz = ox + 1, oy + 1, oz + 1
    code = (sx[:, None, None, :, None, None] * 9 + sy[None, :, None, None, :, None] * 3
            + sz[None, None, :, None, None, :]).reshape(-1, 27)
    return cols, code


def scalar_csr(Nx, Ny, Nz, S, device):
    """(indptr, indices, data) of the scalar operator with stencil S (3,3,3)."""
    n = Nx * Ny * Nz
    cols, code = _pattern(Nx, Ny, Nz, device)
    st = torch.as_tensor(np.asarray(S).reshape(27), dtype=torch.float64, device=device)
    data = st[code].reshape(-1)
    indptr = torch.arange(0, 27 * n + 1, 27, dtype=torch.int64, device=device)
    return indptr, cols.reshape(-1).to(torch.int32), data


def elastic_A_csr(Nx, Ny, Nz, S, device):
    """3n x 3n stiffness: row p + da n, columns q + db n (db blocks in order, q ascending)."""
    n = Nx * Ny * Nz
    cols, code = _pattern(Nx, Ny, Nz, device)
    st = torch.as_tensor(np.asarray(S).reshape(3, 3, 27), dtype=torch.float64, device=device)
    blk = torch.arange(3, device=device, dtype=torch.int64) * n
    col = (cols[None, :, None, :] + blk[None, None, :, None]).expand(3, n, 3, 27).reshape(-1)
    data = st[:, :, code].permute(0, 2, 1, 3).reshape(-1)      # (da, row, db, s)
    indptr = torch.arange(0, 81 * 3 * n + 1, 81, dtype=torch.int64, device=device)
    return indptr, col.to(torch.int32), data


def elastic_F_csr(Nx, Ny, Nz, S, device):
    """3n x 6n coupling: row p + da n, columns 6 q + vb (q ascending, vb inner)."""
    n = Nx * Ny * Nz
    cols, code = _pattern(Nx, Ny, Nz, device)
    st = torch.as_tensor(np.asarray(S).reshape(3, 6, 27), dtype=torch.float64, device=device)
    vb = torch.arange(6, device=device, dtype=torch.int64)
    col = (6 * cols[:, :, None] + vb[None, None, :]).reshape(n, 162)
    col = col[None].expand(3, n, 162).reshape(-1)
    data = st[:, :, code].permute(0, 2, 3, 1).reshape(-1)      # (da, row, s, vb)
    nnz = 3 * n * 162
    indptr = torch.arange(0, nnz + 1, 162, dtype=torch.int64, device=device)
    return indptr, col.to(torch.int32), data


# ------------------------------------------------------------------ modifications
def anchor(indptr, indices, data, anchors, cols_too=True, diag_one=True):
    """Zero anchor rows (and columns), unit anchor diagonal (explicit zeros stay stored)."""
    data = data.clone()
    an = [int(a) for a in anchors]
    for a in an:
        data[int(indptr[a]):int(indptr[a + 1])] = 0.0
    if cols_too:
        data[torch.isin(indices.to(torch.int64), torch.tensor(an, device=data.device))] = 0.0
    if diag_one:
        for a in an:
            s, e = int(indptr[a]), int(indptr[a + 1])
            hit = (indices[s:e] == a).nonzero()
            if hit.numel() != 1:
                raise ValueError("anchor diagonal missing from the pattern")
            data[s + int(hit[0, 0])] = 1.0
    return indptr, indices, data


def _row_ids(indptr, nnz):
    counts = indptr[1:] - indptr[:-1]
    return torch.repeat_interleave(torch.arange(len(counts), device=indptr.device), counts, output_size=nnz)


def drop_defect(indptr, indices, data, defect, cols_too=True, unit_diag=True):
    """Defect enforcement (final_assembly.py:59-158) on a CSR held as tensors."""
    if defect is None or len(defect) == 0:
        return indptr, indices, data
    dev = data.device
    nr = len(indptr) - 1
    isd = torch.zeros(nr if not cols_too else max(nr, int(indices.max()) + 1), dtype=torch.bool, device=dev)
    d = torch.as_tensor(np.asarray(defect), dtype=torch.int64, device=dev)
    isd[d] = True
    rows = _row_ids(indptr, data.numel())
    keep = ~isd[rows]
    if cols_too:
        keep &= ~isd[indices.to(torch.int64)]
    cnt = torch.bincount(rows[keep], minlength=nr)
    if unit_diag:
        cnt[d] = 1
    new_ptr = torch.zeros(nr + 1, dtype=torch.int64, device=dev)
    new_ptr[1:] = torch.cumsum(cnt, 0)
    kr = rows[keep]
    kc = torch.bincount(kr, minlength=nr)
    kcum = torch.cumsum(kc, 0) - kc
    pos = new_ptr[kr] + (torch.arange(kr.numel(), device=dev) - kcum[kr])
    new_idx = torch.empty(int(new_ptr[-1]), dtype=torch.int32, device=dev)
    new_val = torch.empty(int(new_ptr[-1]), dtype=torch.float64, device=dev)
    new_idx[pos] = indices[keep]
    new_val[pos] = data[keep]
    if unit_diag:
        new_idx[new_ptr[d]] = d.to(torch.int32)
        new_val[new_ptr[d]] = 1.0
    return new_ptr, new_idx, new_val
