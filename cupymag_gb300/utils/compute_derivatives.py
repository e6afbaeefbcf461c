"""Gradients from the F matrices (drop-in for cupymag/utils/compute_derivatives.py:19-125).

Fx, Fy, Fz share one sparsity pattern, so both operators run as single
kernels that read the pattern once:
* compute_Hd_from_U: Hd_i = -F_i U for i = x, y, z (:36-58);
* compute_E_from_u: Voigt strain from the nine products D_a u_b, optionally
  rotated by R (:60-125).
"""
from __future__ import annotations

import torch

from .. import _native as N
from .device_csr import DeviceCSR


class ComputeDerivatives:
    def __init__(self, Fx: DeviceCSR, Fy: DeviceCSR, Fz: DeviceCSR):
        if not (Fx.same_pattern(Fy) and Fx.same_pattern(Fz)):
            raise ValueError("Fx, Fy, Fz must share one sparsity pattern")
        self.Dx, self.Dy, self.Dz = Fx, Fy, Fz
        self._R = {}

    def hd_into(self, U, out):
        N.check(N.lib().cpm_spmv_csr_multi(self.Dx.struct(), self.Dy.data.data_ptr(), self.Dz.data.data_ptr(),
                                           U.data_ptr(), out.data_ptr(), -1.0, 0, None, -1, N.stream_ptr()),
                "cpm_spmv_csr_multi")
        return out

    def demag_rhs_into(self, m, avg_m, out, pin=0):
        """b = -(Fx (m_x - <m>_x) + Fy (...) + Fz (...)), b[pin] = 0 (Micromagnetics.py:166-168)."""
        N.check(N.lib().cpm_spmv_csr_multi(self.Dx.struct(), self.Dy.data.data_ptr(), self.Dz.data.data_ptr(),
                                           m.data_ptr(), out.data_ptr(), -1.0, 1,
                                           None if avg_m is None else avg_m.data_ptr(), int(pin), N.stream_ptr()),
                "cpm_spmv_csr_multi")
        return out

    def compute_Hd_from_U(self, U):
        U = torch.as_tensor(U, dtype=torch.float64, device=self.Dx.device).contiguous()
        out = torch.empty((U.shape[0], 3), dtype=torch.float64, device=U.device)
        self.hd_into(U, out)
        return out[:, 0], out[:, 1], out[:, 2]

    def _R9(self, R):
        if R is None:
            return None
        key = tuple(float(v) for v in torch.as_tensor(R).reshape(-1).tolist())
        if key not in self._R:
            self._R[key] = torch.tensor(key, dtype=torch.float64, device=self.Dx.device)
        return self._R[key]

    def strain_into(self, u, out, R9=None):
        N.check(N.lib().cpm_strain_from_u(self.Dx.struct(), self.Dy.data.data_ptr(), self.Dz.data.data_ptr(),
                                          u.data_ptr(), None if R9 is None else R9.data_ptr(), out.data_ptr(),
                                          N.stream_ptr()), "cpm_strain_from_u")
        return out

    def compute_E_from_u(self, n, u, R=None):
        u = torch.as_tensor(u, dtype=torch.float64, device=self.Dx.device).contiguous()
        if u.numel() != 3 * n or self.Dx.shape[0] != n:
            raise ValueError("u must hold 3 n values [ux|uy|uz]")
        out = torch.empty((n, 6), dtype=torch.float64, device=u.device)
        return self.strain_into(u, out, self._R9(R))
