"""Rotation matrices for the crystal x-axis along [111] (cupymag/utils/rot_111_matrices.py:21-103).

R (3x3) maps x -> [111]; M (6x6) rotates Voigt strains/stiffness accordingly.
``backend`` is "numpy" (default) or "torch"; the reference's "cupy" is
accepted as an alias of "torch" (device arrays).
"""
import numpy as np

from ..core.constants import inv_sqrt2, inv_sqrt3, inv_sqrt6, sqrt2, sqrt3


def _as(arr, backend, dtype):
    if backend == "numpy":
        return np.asarray(arr, dtype=dtype or np.float64)
    if backend in ("torch", "cupy"):
        import torch
        return torch.tensor(arr, dtype=dtype or torch.float64, device="cuda")
    raise ValueError("Backend must be 'numpy' or 'torch'")


def get_R_matrix(backend="numpy", dtype=None):
    R = [[inv_sqrt3, inv_sqrt3, inv_sqrt3],
         [-inv_sqrt2, inv_sqrt2, 0.0],
         [-inv_sqrt6, -inv_sqrt6, 2 * inv_sqrt6]]
    return _as(R, backend, dtype)


def get_M_matrix(backend="numpy", dtype=None):
    M = [[1 / 3, 1 / 3, 1 / 3, 2 / 3, 2 / 3, 2 / 3],
         [1 / 2, 1 / 2, 0.0, 0.0, 0.0, -1.0],
         [1 / 6, 1 / 6, 2 / 3, -2 / 3, -2 / 3, 1 / 3],
         [sqrt3 / 6, -sqrt3 / 6, 0.0, sqrt3 / 3, -sqrt3 / 3, 0.0],
         [-sqrt2 / 6, -sqrt2 / 6, sqrt2 / 3, sqrt2 / 6, sqrt2 / 6, -sqrt2 / 3],
         [-inv_sqrt6, inv_sqrt6, 0.0, inv_sqrt6, -inv_sqrt6, 0.0]]
    return _as(M, backend, dtype)
