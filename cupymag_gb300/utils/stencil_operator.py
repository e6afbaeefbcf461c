"""Matrix-free periodic hex operators (see csrc/stencil.cu).

A ``StencilOperator`` holds the 27-point coefficients of one structured hex
operator (exactly the values of its CSR rows) plus per-DOF flags for the
anchor and defect rows/columns, and applies it through the C-ABI
(``cpm_stencil_apply``, ``cpm_cg_solve_stencil``) without a matrix stream.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _native as N

ROW_IDENTITY, ROW_ZERO, COL_EXCLUDED, NEAR_EXCLUDED, NEAR_UNPINNED = 1, 2, 4, 8, 16


class StencilOperator:
    def __init__(self, nx, ny, nz, coef, flags=None, device=None):
        self.nx, self.ny, self.nz = int(nx), int(ny), int(nz)
        coef = np.asarray(coef, dtype=np.float64).reshape(-1)
        self.ncomp = {27: 1, 243: 3}[coef.size]
        dev = device or torch.device("cuda", torch.cuda.current_device())
        self.coef_host = coef.copy()
        self._dev = torch.device(dev)
        self.n = self.nx * self.ny * self.nz
        # the one node whose rows and columns the operator pins (the reference's anchor), or -1
        self.anchor = -1
        if flags is not None:
            flags = self.mark_neighbours(np.asarray(flags, dtype=np.uint8).copy())
            marked = np.flatnonzero(flags & 7)
            if marked.size == 1 and (flags[marked[0]] & 7) == (ROW_IDENTITY | COL_EXCLUDED):
                self.anchor = int(marked[0])
        self.flags = None if flags is None else torch.as_tensor(flags, device=dev)
        self.shape = (self.n * self.ncomp, self.n * self.ncomp)
        self._struct = None

    @property
    def device(self):
        return self._dev

    def mark_neighbours(self, f):
        """Set NEAR_EXCLUDED on every DOF that has an excluded column among its 27 neighbours, and
        NEAR_UNPINNED where one of those excluded columns is not also an identity row."""
        shape = (self.nx, self.ny, self.nz)
        ex = (f & COL_EXCLUDED).astype(bool).reshape(shape)
        unpinned = ex & ~(f & ROW_IDENTITY).astype(bool).reshape(shape)

        def near(m):
            out = np.zeros_like(m)
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        out |= np.roll(m, (dx, dy, dz), axis=(0, 1, 2))
            return out.reshape(-1)

        f[near(ex)] |= NEAR_EXCLUDED
        if unpinned.any():
            f[near(unpinned)] |= NEAR_UNPINNED
        return f

    def ensure_fp32(self):
        return self

    def struct(self) -> N.Stencil:
        if self._struct is None:
            s = N.Stencil()
            s.nx, s.ny, s.nz, s.ncomp = self.nx, self.ny, self.nz, self.ncomp
            s.coef[:self.coef_host.size] = tuple(float(v) for v in self.coef_host)
            s.flags = None if self.flags is None else self.flags.data_ptr()
            self._struct = s
        return self._struct

    def spmv(self, x: torch.Tensor, out: torch.Tensor = None, alpha: float = 1.0) -> torch.Tensor:
        x = x.contiguous()
        nvec = 1 if x.dim() == 1 else x.shape[1]
        if x.shape[0] != self.shape[1] or nvec not in (1, 3) or (self.ncomp == 3 and nvec != 1):
            raise ValueError(f"shape mismatch: {self.shape} @ {tuple(x.shape)}")
        if out is None:
            out = torch.empty_like(x)
        N.check(N.lib().cpm_stencil_apply(self.struct(), x.data_ptr(), out.data_ptr(), float(alpha), nvec,
                                          N.stream_ptr()), "cpm_stencil_apply")
        return out

    def spmv32(self, x: torch.Tensor, form: int = 2, out: torch.Tensor = None) -> torch.Tensor:
        """y = A x in FP32 (the refinement form's product); form 0 per DOF, 1 aligned quads, 2 scalar-load quads."""
        x = x.contiguous()
        nvec = 1 if x.dim() == 1 else x.shape[1]
        if x.dtype != torch.float32 or x.shape[0] != self.shape[1] or nvec not in (1, 3) or \
                (self.ncomp == 3 and nvec != 1):
            raise ValueError(f"shape/dtype mismatch: {self.shape} @ {tuple(x.shape)} {x.dtype}")
        if out is None:
            out = torch.empty_like(x)
        N.check(N.lib().cpm_stencil_apply32(self.struct(), x.data_ptr(), out.data_ptr(), nvec, int(form),
                                            N.stream_ptr()), "cpm_stencil_apply32")
        return out

    def __matmul__(self, x):
        return self.spmv(x)

    def fft_plan(self, layout: int = N.FFT_LAYOUT_AUTO):
        """The circulant-inverse preconditioner of this operator in the given spectrum layout
        (N.FFT_LAYOUT_*; built once per layout; None when the grid's dimensions are not supported)."""
        plans = self.__dict__.setdefault("_fft", {})
        if layout not in plans:
            nb = int(N.lib().cpm_fft_precond_bytes(self.nx, self.ny, self.nz, self.ncomp))
            if nb <= 0:
                return None
            mem = torch.empty(nb, dtype=torch.uint8, device=self.device)
            if mem.data_ptr() % 256:
                raise RuntimeError("plan memory is not 256-byte aligned")
            plan = N.FftPrecondC()
            plan.layout = int(layout)
            plan.anchor = self.anchor
            N.check(N.lib().cpm_fft_precond_build(self.struct(), mem.data_ptr(), nb, plan, N.stream_ptr()),
                    "cpm_fft_precond_build")
            plans[layout] = (plan, mem)
        return plans[layout][0]

    def precondition32(self, r: torch.Tensor, out: torch.Tensor = None,
                       layout: int = N.FFT_LAYOUT_AUTO) -> torch.Tensor:
        """z = M r with M the circulant-inverse preconditioner (FP32), as the preconditioned solve applies it."""
        plan = self.fft_plan(layout)
        if plan is None:
            raise ValueError(f"no FFT preconditioner for a {self.nx} x {self.ny} x {self.nz} grid")
        r = r.contiguous()
        if r.dtype != torch.float32 or r.numel() != self.shape[0]:
            raise ValueError("r must be a float32 vector of the operator's size")
        out = torch.empty_like(r) if out is None else out
        work = torch.empty(8 * r.numel(), dtype=torch.uint8, device=r.device)
        N.check(N.lib().cpm_fft_precond_apply(plan, r.data_ptr(), out.data_ptr(), work.data_ptr(), work.numel(),
                                              N.stream_ptr()), "cpm_fft_precond_apply")
        return out

    # the same operator with unit (and excluded) rows at the given DOFs
    @staticmethod
    def flags_for(n, dofs, bits):
        f = np.zeros(n, dtype=np.uint8)
        f[np.asarray(dofs, dtype=np.int64)] = bits
        return f
