"""Host -> device handoff of assembled matrices and the eigenstrain
(drop-in for cupymag/utils/final_assembly.py:27-266)."""
from __future__ import annotations

import numpy as np
import torch

from .. import _native as N
from ..mesh.grids import extract_defect_dofs  # noqa: F401  (same name as the reference)
from ..physics.assembly import enforce_defect_A, enforce_defect_F, to_csr
from .device_csr import DeviceCSR


def enforce_defect_region_A(A, defect_dofs=None):
    """final_assembly.py:59-111 on a SciPy CSR."""
    return enforce_defect_A(A, None if defect_dofs is None else np.asarray(defect_dofs))


def enforce_defect_region_F(F, defect_dofs=None):
    """final_assembly.py:114-158 on a SciPy CSR."""
    return enforce_defect_F(F, None if defect_dofs is None else np.asarray(defect_dofs))


def assemble_stiffness_matrix(rows_np, cols_np, vals_np, nDOFx, defect_dofs=None, nDOFy=None):
    """COO -> CSR (duplicates summed), defect rows/columns -> identity, upload (final_assembly.py:160-181)."""
    A = to_csr(rows_np, cols_np, vals_np, (nDOFx, nDOFy or nDOFx))
    return DeviceCSR.from_scipy(enforce_defect_region_A(A, defect_dofs))


def assemble_mass_matrix(rows_np, cols_np, vals_np, nDOFx, defect_dofs=None, nDOFy=None):
    """COO -> CSR, defect rows dropped, upload (final_assembly.py:184-205)."""
    F = to_csr(rows_np, cols_np, vals_np, (nDOFx, nDOFy or nDOFx))
    return DeviceCSR.from_scipy(enforce_defect_region_F(F, defect_dofs))


def build_E0_from_m(lam100, lam111, m_nodes, out=None, R9=None, M36=None):
    """Eigenstrain (6n,) node-interleaved [exx, eyy, ezz, 2exy, 2eyz, 2exz] (final_assembly.py:208-266)."""
    m = torch.as_tensor(m_nodes, dtype=torch.float64, device="cuda").contiguous()
    if m.dim() == 1:
        m = m.reshape(-1, 3)
    n = m.shape[0]
    if out is None:
        out = torch.empty(6 * n, dtype=torch.float64, device=m.device)
    N.check(N.lib().cpm_build_E0(n, m.data_ptr(), float(lam100), float(lam111),
                                 None if R9 is None else R9.data_ptr(), None if M36 is None else M36.data_ptr(),
                                 out.data_ptr(), N.stream_ptr()), "cpm_build_E0")
    return out
