"""Precision names (cupymag/utils/precision_select.py:16-53).

"DP" selects the plain FP64 method.  "SP" in the reference runs everything in
FP32; here it (and "IR") selects FP32 CG inside FP64 iterative refinement, which
stops on the same FP64 residual test as "DP".
"""
import numpy as np


def get_float_type(precision: str, backend: str = "numpy"):
    if precision not in ("SP", "DP", "IR"):
        raise ValueError(f"Invalid precision '{precision}'. Choose 'SP', 'DP' or 'IR'.")
    if backend == "numpy":
        return np.float64
    if backend in ("torch", "cupy"):
        import torch
        return torch.float64
    raise ValueError(f"Unsupported backend '{backend}'. Choose 'numpy' or 'torch'.")


def solver_precision(precision: str) -> str:
    return "DP" if precision == "DP" else "IR"
