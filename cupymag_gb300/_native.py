"""ctypes binding of ``libcupymag_gb300.so`` (the C-ABI of include/cupymag_gb300.h).

The library is built in-tree by ``cupymag_gb300.build``.  There is no fallback:
if the library is missing or no CUDA device is present, every device entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import threading

from .build import LIB

_lock = threading.Lock()
_lib = None

CPM_OK, CPM_NOT_CONVERGED, CPM_BARRIER_TIMEOUT, CPM_NONFINITE, CPM_BAD_ARG, CPM_CUDA_ERROR = range(6)
# iteration forms of the FP32 stencil CG (cpm_cg_opts.form)
CG_FORM_DEFAULT, CG_FORM_THREE_BARRIER, CG_FORM_TWO_BARRIER, CG_FORM_FFT_PCG = 0, 1, 2, 3
# spectrum layouts of the FFT preconditioner (cpm_fft_precond.layout)
FFT_LAYOUT_AUTO, FFT_LAYOUT_SLAB, FFT_LAYOUT_PASSES = 0, 1, 2
STATUS_NAMES = {0: "ok", 1: "not converged", 2: "grid barrier timeout", 3: "non-finite value", 4: "bad argument",
                5: "CUDA error"}

vp = C.c_void_p
i64 = C.c_int64
i32 = C.c_int32
dbl = C.c_double


class CSR(C.Structure):
    _fields_ = [("rows", i64), ("cols", i64), ("nnz", i64), ("indptr", vp), ("indptr_is64", i32),
                ("indices", vp), ("vals", vp), ("vals32", vp), ("max_row_nnz", i64)]


class Stencil(C.Structure):
    _fields_ = [("nx", i32), ("ny", i32), ("nz", i32), ("ncomp", i32), ("coef", dbl * 243), ("flags", vp)]


class CGInfo(C.Structure):
    _fields_ = [("status", i32), ("iters", i32 * 3), ("outer", i32), ("df_updates", i32), ("resid", dbl * 3),
                ("bnorm", dbl * 3)]


class CGOpts(C.Structure):
    _fields_ = [("tol", dbl), ("maxiter", i32), ("use_init_host", i32), ("use_init_dev", vp), ("precision", i32),
                ("inner_tol", dbl), ("max_outer", i32), ("form", i32), ("barrier_timeout_s", dbl),
                ("carry_b", vp), ("carry_t", vp), ("carry_valid", vp)]


class FieldParams(C.Structure):
    _fields_ = [("K1", dbl), ("elasC1", dbl), ("elasC2", dbl), ("elasC3", dbl), ("lambda100", dbl),
                ("Nd", dbl * 3), ("Hext", dbl * 3), ("R", dbl * 9), ("rot111", i32), ("has_E", i32),
                ("hext_sched", vp), ("hext_step", vp)]


class BatchSystem(C.Structure):
    _fields_ = [("nx", i32), ("ny", i32), ("nz", i32), ("maxiter", i32), ("tol", dbl), ("flags", vp), ("b", vp),
                ("x", vp), ("use_init_dev", vp), ("info", vp), ("work", vp)]


class BatchPlan(C.Structure):
    _fields_ = [("dev", vp), ("bytes", i64), ("nsys", i32), ("grid", i32), ("ncomp", i32), ("nrhs", i32),
                ("precision", i32), ("total_chunks", i32), ("coef", dbl * 243)]


class DerivStencilC(C.Structure):
    _fields_ = [("nx", i32), ("ny", i32), ("nz", i32), ("pad", i32), ("fx", dbl * 27), ("fy", dbl * 27),
                ("fz", dbl * 27)]


class FelStencilC(C.Structure):
    _fields_ = [("nx", i32), ("ny", i32), ("nz", i32), ("anchor", i32), ("coef", dbl * 486)]


class FftPrecondC(C.Structure):
    _fields_ = [("nx", i32), ("ny", i32), ("nz", i32), ("ncomp", i32), ("dev", vp), ("bytes", i64),
                ("npass", i32 * 3), ("radix", (i32 * 16) * 3), ("layout", i32), ("anchor", i32)]


CG_INFO_BYTES = C.sizeof(CGInfo)

_PROTOS = {
    "cpm_version": (C.c_char_p, []),
    "cpm_last_error_string": (C.c_char_p, []),
    "cpm_device_sm_count": (C.c_int, [C.c_int]),
    "cpm_spmv_csr": (C.c_int, [C.POINTER(CSR), vp, vp, dbl, C.c_int, vp]),
    "cpm_spmv_csr_multi": (C.c_int, [C.POINTER(CSR), vp, vp, vp, vp, dbl, C.c_int, vp, i64, vp]),
    "cpm_cg_workspace_bytes": (C.c_size_t, [i64, C.c_int, C.c_int]),
    "cpm_cg_stencil_workspace_bytes": (C.c_size_t, [i64, C.c_int, C.c_int]),
    "cpm_stencil_df_error_bound": (C.c_double, [C.POINTER(Stencil)]),
    "cpm_cg_solve": (C.c_int, [C.POINTER(CSR), vp, vp, C.c_int, C.POINTER(CGOpts), vp, C.c_size_t, vp, vp]),
    "cpm_cg_solve_noalloc": (C.c_int, [C.POINTER(CSR), vp, vp, C.c_int, C.POINTER(CGOpts), vp, vp]),
    "cpm_stencil_apply": (C.c_int, [C.POINTER(Stencil), vp, vp, dbl, C.c_int, vp]),
    "cpm_stencil_apply32": (C.c_int, [C.POINTER(Stencil), vp, vp, C.c_int, C.c_int, vp]),
    "cpm_cg_solve_stencil": (C.c_int, [C.POINTER(Stencil), vp, vp, C.c_int, C.POINTER(CGOpts), vp, C.c_size_t, vp,
                                       vp]),
    "cpm_batch_work_bytes": (i64, [i32, i32, i32, i32, i32, i32]),
    "cpm_batch_plan_bytes": (C.c_int, [C.POINTER(BatchSystem), i32, i32, i32, i32, C.POINTER(i64)]),
    "cpm_batch_plan_build": (C.c_int, [C.POINTER(BatchSystem), i32, i32, i32, i32, vp, vp, i64, C.POINTER(BatchPlan),
                                       vp]),
    "cpm_cg_solve_blockdiag": (C.c_int, [C.POINTER(BatchPlan), C.POINTER(CGOpts), vp]),
    "cpm_record_step": (C.c_int, [vp, vp, vp, vp, i32, vp]),
    "cpm_coo_segment_sum": (C.c_int, [vp, vp, i64, vp, vp]),
    "cpm_llg_field": (C.c_int, [C.POINTER(FieldParams), i64, vp, vp, vp, vp, dbl, vp, vp, vp]),
    "cpm_gs_star": (C.c_int, [C.c_int, i64, vp, vp, vp, vp, vp, dbl, vp, vp, vp]),
    "cpm_renorm_sumsq": (C.c_int, [i64, vp, vp, vp, vp, vp, dbl, dbl, vp, vp, vp, vp, vp]),
    "cpm_volavg_scratch_doubles": (C.c_size_t, [C.c_int]),
    "cpm_volavg": (C.c_int, [i64, C.c_int, vp, vp, dbl, vp, vp, vp, vp]),
    "cpm_build_E0": (C.c_int, [i64, vp, dbl, dbl, vp, vp, vp, vp]),
    "cpm_strain_from_u": (C.c_int, [C.POINTER(CSR), vp, vp, vp, vp, vp, vp]),
    "cpm_strain_finalize": (C.c_int, [i64, vp, vp, vp, dbl, dbl, vp, vp, vp, C.c_int, vp]),
    "cpm_stencil_deriv": (C.c_int, [C.POINTER(DerivStencilC), vp, vp, dbl, C.c_int, vp, i64, vp]),
    "cpm_stencil_strain": (C.c_int, [C.POINTER(DerivStencilC), vp, vp, vp, vp]),
    "cpm_stencil_fel": (C.c_int, [C.POINTER(FelStencilC), vp, vp, vp]),
    "cpm_fft_precond_bytes": (i64, [i32, i32, i32, i32]),
    "cpm_fft_precond_build": (C.c_int, [C.POINTER(Stencil), vp, i64, C.POINTER(FftPrecondC), vp]),
    "cpm_fft_precond_apply": (C.c_int, [C.POINTER(FftPrecondC), vp, vp, vp, i64, vp]),
    "cpm_cg_fft_workspace_bytes": (C.c_size_t, [i32, i32, i32, i32]),
    "cpm_cg_solve_stencil_fft": (C.c_int, [C.POINTER(Stencil), C.POINTER(FftPrecondC), vp, vp, C.POINTER(CGOpts),
                                           vp, C.c_size_t, vp, vp]),
}

EXPORTED = tuple(_PROTOS)


def load(build_if_missing: bool = False):
    """Load the shared library (optionally building it first)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        import torch  # noqa: F401  (libcudart is resolved from the already-loaded torch)
        if not LIB.exists():
            if build_if_missing:
                from .build import build
                build()
            else:
                raise RuntimeError(
                    f"cupymag_gb300 native library not found at {LIB}; build it with "
                    "`python -m cupymag_gb300.build` (needs nvcc from CUDA 13)")
        lib = C.CDLL(str(LIB), mode=C.RTLD_GLOBAL)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def lib():
    return _lib if _lib is not None else load()


def last_error() -> str:
    return lib().cpm_last_error_string().decode(errors="replace")


def check(status: int, what: str):
    if status != CPM_OK:
        raise RuntimeError(f"{what} failed ({STATUS_NAMES.get(status, status)}): {last_error()}")


def require_cuda():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("cupymag_gb300 needs a CUDA GPU (GB300, sm_103a); no CUDA device is available")


def stream_ptr(stream=None) -> int:
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return s.cuda_stream
