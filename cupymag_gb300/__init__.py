"""cupymag_gb300: GB300-native (sm_103a) Gauss-Seidel-projection LLG step for CuPyMag.

Host code is Python; the hot path (persistent fused CG, CSR SpMV, effective
field, Gauss-Seidel projection, renormalisation, volume averages) runs in the
hand-written CUDA kernels of ``libcupymag_gb300.so`` through a C-ABI
(include/cupymag_gb300.h).  PyTorch tensors own the device memory.
"""
__version__ = "0.9.1+gb300.1"

REFERENCE_VERSION = "0.9.1"
