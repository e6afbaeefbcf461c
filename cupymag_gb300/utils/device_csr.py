"""CSR matrices resident in GPU memory (torch tensors), handed to the C-ABI.

This is the device side of the reference's host->device handoff
(cupymag/utils/final_assembly.py:160-205, ``cpx.csr_matrix(A_scipy)``): the
SciPy CSR from assembly is uploaded once; index arrays are int32 (row
pointers int64 when nnz >= 2^31), values FP64, plus an optional FP32 copy of
the values for the mixed-precision solver.  ``A @ x`` runs the library's SpMV.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import torch

from .. import _native as N


def validate_csr(A: sp.csr_matrix):
    """Host-side structural checks before upload (row pointers monotone, columns in range)."""
    ip = A.indptr
    if ip[0] != 0 or ip[-1] != A.nnz or np.any(np.diff(ip) < 0):
        raise ValueError("CSR row pointers are not monotone from 0 to nnz")
    if A.nnz and (A.indices.min() < 0 or A.indices.max() >= A.shape[1]):
        raise ValueError("CSR column index out of range")
    if A.shape[1] > np.iinfo(np.int32).max:
        raise ValueError("column count exceeds int32 indices")


class DeviceCSR:
    def __init__(self, indptr: torch.Tensor, indices: torch.Tensor, data: torch.Tensor, shape, data32=None):
        self.indptr = indptr
        self.indices = indices
        self.data = data
        self.data32 = data32
        self.shape = (int(shape[0]), int(shape[1]))
        self._struct = None

    @classmethod
    def from_scipy(cls, A, device=None, fp32=False, validate=True):
        A = sp.csr_matrix(A)
        if not A.has_sorted_indices:
            A.sort_indices()
        if validate:
            validate_csr(A)
        dev = device or torch.device("cuda", torch.cuda.current_device())
        big = A.nnz >= 2 ** 31
        ip = torch.from_numpy(np.ascontiguousarray(A.indptr, dtype=np.int64 if big else np.int32)).to(dev)
        ci = torch.from_numpy(np.ascontiguousarray(A.indices, dtype=np.int32)).to(dev)
        va = torch.from_numpy(np.ascontiguousarray(A.data, dtype=np.float64)).to(dev)
        obj = cls(ip, ci, va, A.shape)
        if fp32:
            obj.ensure_fp32()
        return obj

    def ensure_fp32(self):
        if self.data32 is None:
            self.data32 = self.data.to(torch.float32)
            self._struct = None
        return self

    @property
    def max_row_nnz(self) -> int:
        if getattr(self, "_max_row", None) is None:
            self._max_row = int((self.indptr[1:] - self.indptr[:-1]).max().item()) if self.shape[0] else 0
        return self._max_row

    @property
    def nnz(self) -> int:
        return int(self.data.numel())

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def device(self):
        return self.data.device

    def nbytes(self, fp32=False) -> int:
        vals = self.nnz * (4 if fp32 else 8)
        return vals + self.indices.numel() * 4 + self.indptr.numel() * self.indptr.element_size()

    def struct(self) -> N.CSR:
        if self._struct is None:
            s = N.CSR()
            s.rows, s.cols, s.nnz = self.shape[0], self.shape[1], self.nnz
            s.indptr = self.indptr.data_ptr()
            s.indptr_is64 = 1 if self.indptr.dtype == torch.int64 else 0
            s.indices = self.indices.data_ptr()
            s.vals = self.data.data_ptr()
            s.vals32 = self.data32.data_ptr() if self.data32 is not None else None
            s.max_row_nnz = self.max_row_nnz
            self._struct = s
        return self._struct

    def spmv(self, x: torch.Tensor, out: torch.Tensor = None, alpha: float = 1.0) -> torch.Tensor:
        x = x.contiguous()
        if x.dtype != torch.float64 or x.device != self.device:
            raise TypeError("DeviceCSR @ x needs a float64 tensor on the matrix's device")
        nvec = 1 if x.dim() == 1 else x.shape[1]
        if x.shape[0] != self.shape[1] or nvec not in (1, 3):
            raise ValueError(f"shape mismatch: {self.shape} @ {tuple(x.shape)}")
        if out is None:
            out = torch.empty((self.shape[0],) if nvec == 1 else (self.shape[0], nvec), dtype=torch.float64,
                              device=self.device)
        N.check(N.lib().cpm_spmv_csr(self.struct(), x.data_ptr(), out.data_ptr(), float(alpha), nvec,
                                     N.stream_ptr()), "cpm_spmv_csr")
        return out

    def __matmul__(self, x):
        return self.spmv(x)

    def __neg__(self):
        return DeviceCSR(self.indptr, self.indices, -self.data, self.shape,
                         None if self.data32 is None else -self.data32)

    def to_scipy(self) -> sp.csr_matrix:
        return sp.csr_matrix((self.data.cpu().numpy(), self.indices.cpu().numpy(), self.indptr.cpu().numpy()),
                             shape=self.shape)

    def same_pattern(self, other: "DeviceCSR") -> bool:
        return (self.shape == other.shape and self.nnz == other.nnz and torch.equal(self.indptr, other.indptr)
                and torch.equal(self.indices, other.indices))
