"""Precision names (cupymag/utils/precision_select.py:16-53).

``get_float_type`` returns what the reference returns: float32 for "SP" and
float64 for "DP", for NumPy and for the device backend (torch here, CuPy in
the reference).  This package adds "IR", its precision form, whose stored
state stays FP64 (float64).

The config's ``precision`` selects the solver form through
``solver_precision``: "DP" is the plain FP64 method; "SP" and "IR" both run
the CG solves in FP32 inside FP64 iterative refinement, which stops on the
same FP64 residual test as "DP".  The reference's "SP" runs every array in
FP32; this package never stores m, u or the fields in FP32, so an "SP" config
gets the refinement form (at least as accurate as the reference's SP run).
"""
import numpy as np


def get_float_type(precision: str, backend: str = "numpy"):
    if precision not in ("SP", "DP", "IR"):
        raise ValueError(f"Invalid precision '{precision}'. Choose 'SP', 'DP' or 'IR'.")
    single = precision == "SP"
    if backend == "numpy":
        return np.float32 if single else np.float64
    if backend in ("torch", "cupy"):
        import torch
        return torch.float32 if single else torch.float64
    if backend == "numba":
        raise ImportError("Backend 'numba' could not be imported. Make sure it's installed.")
    raise ValueError(f"Unsupported backend '{backend}'. Choose 'numpy', 'cupy' (torch here), or 'numba'.")


def solver_precision(precision: str) -> str:
    """The solver form a config's precision selects: "DP" plain FP64, anything else FP32 + FP64 refinement."""
    return "DP" if precision == "DP" else "IR"
