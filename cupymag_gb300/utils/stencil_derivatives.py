"""Matrix-free derivative and coupling operators of structured hex grids (see csrc/deriv.cu).

``StencilDerivatives`` is the drop-in for ``ComputeDerivatives``
(cupymag/utils/compute_derivatives.py:19-125) when Fx, Fy, Fz are the
27-point stencils of a grid of identical unit cells: Hd = -F U, the demag
right-hand side, and the strain from u, with no CSR matrix in memory.
``StencilCoupling`` applies F_el (cupymag/physics/assemble_elasticity.py:268-459)
the same way: b_el = F_el E0 (cupymag/core/Micromagnetics.py:123).
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _native as N


class StencilDerivatives:
    def __init__(self, nx, ny, nz, fx, fy, fz, device=None):
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.n = self.nx * self.ny * self.nz
        self.coef = [np.asarray(f, dtype=np.float64).reshape(27).copy() for f in (fx, fy, fz)]
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.shape = (self.n, self.n)
        self._struct = None
        self._R = {}

    def struct(self) -> N.DerivStencilC:
        if self._struct is None:
            s = N.DerivStencilC()
            s.nx, s.ny, s.nz = self.nx, self.ny, self.nz
            s.fx[:], s.fy[:], s.fz[:] = (tuple(float(v) for v in c) for c in self.coef)
            self._struct = s
        return self._struct

    def nbytes(self) -> int:
        return 0   # the coefficients travel with each launch

    def hd_into(self, U, out):
        """out (n,3) = -(Fx U, Fy U, Fz U)  (compute_derivatives.py:36-58)."""
        N.check(N.lib().cpm_stencil_deriv(self.struct(), U.data_ptr(), out.data_ptr(), -1.0, 0, None, -1,
                                          N.stream_ptr()), "cpm_stencil_deriv")
        return out

    def demag_rhs_into(self, m, avg_m, out, pin=0):
        """b = -(Fx (m_x - <m>_x) + Fy (...) + Fz (...)), b[pin] = 0 (Micromagnetics.py:166-168)."""
        N.check(N.lib().cpm_stencil_deriv(self.struct(), m.data_ptr(), out.data_ptr(), -1.0, 1,
                                          None if avg_m is None else avg_m.data_ptr(), int(pin), N.stream_ptr()),
                "cpm_stencil_deriv")
        return out

    def compute_Hd_from_U(self, U):
        U = torch.as_tensor(U, dtype=torch.float64, device=self.device).contiguous()
        out = torch.empty((U.shape[0], 3), dtype=torch.float64, device=U.device)
        self.hd_into(U, out)
        return out[:, 0], out[:, 1], out[:, 2]

    def _R9(self, R):
        if R is None:
            return None
        key = tuple(float(v) for v in torch.as_tensor(R).reshape(-1).tolist())
        if key not in self._R:
            self._R[key] = torch.tensor(key, dtype=torch.float64, device=self.device)
        return self._R[key]

    def strain_into(self, u, out, R9=None):
        N.check(N.lib().cpm_stencil_strain(self.struct(), u.data_ptr(), None if R9 is None else R9.data_ptr(),
                                           out.data_ptr(), N.stream_ptr()), "cpm_stencil_strain")
        return out

    def compute_E_from_u(self, n, u, R=None):
        u = torch.as_tensor(u, dtype=torch.float64, device=self.device).contiguous()
        if u.numel() != 3 * n or self.n != n:
            raise ValueError("u must hold 3 n values [ux|uy|uz]")
        out = torch.empty((n, 6), dtype=torch.float64, device=u.device)
        return self.strain_into(u, out, self._R9(R))


class StencilCoupling:
    """F_el (3n x 6n) as a stencil with 3 x 6 coefficient blocks; rows of DOF 0 empty (the anchors)."""

    def __init__(self, nx, ny, nz, coef, anchor=True, device=None):
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        self.n = self.nx * self.ny * self.nz
        self.coef = np.asarray(coef, dtype=np.float64).reshape(486).copy()
        self.anchor = bool(anchor)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.shape = (3 * self.n, 6 * self.n)
        self._struct = None

    def struct(self) -> N.FelStencilC:
        if self._struct is None:
            s = N.FelStencilC()
            s.nx, s.ny, s.nz, s.anchor = self.nx, self.ny, self.nz, 1 if self.anchor else 0
            s.coef[:] = tuple(float(v) for v in self.coef)
            self._struct = s
        return self._struct

    def nbytes(self) -> int:
        return 0

    def spmv(self, x: torch.Tensor, out: torch.Tensor = None) -> torch.Tensor:
        x = x.contiguous()
        if x.dim() != 1 or x.shape[0] != self.shape[1] or x.dtype != torch.float64:
            raise ValueError(f"F_el @ x needs a float64 vector of {self.shape[1]} values")
        if out is None:
            out = torch.empty(self.shape[0], dtype=torch.float64, device=x.device)
        N.check(N.lib().cpm_stencil_fel(self.struct(), x.data_ptr(), out.data_ptr(), N.stream_ptr()),
                "cpm_stencil_fel")
        return out

    def __matmul__(self, x):
        return self.spmv(x)
