"""Conjugate-gradient solves on the GPU (drop-in for cupymag/solvers/linear_solvers.py).

``solve_cg`` keeps the reference signature and behaviour
(linear_solvers.py:20-74): x0 is used only when ``use_init`` is true, the
tolerance is relative to ||b||, a zero right-hand side returns b, and a solve
that reaches ``maxiter`` raises ``RuntimeError`` with the same message text
("Error! CG for {system} did not converge. info={info}, residual={rnorm}.").

The work runs in one persistent cooperative kernel per solve (see
csrc/cg.cu).  ``CGSolver`` keeps the workspace between solves so the LLG step
allocates nothing per step; ``precision="IR"`` selects FP32 CG inside FP64
iterative refinement.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .. import _native as N
from ..utils.device_csr import DeviceCSR

PRECISIONS = {"DP": 0, "FP64": 0, "IR": 1, "MIXED": 1, "SP": 1}


class CGSolver:
    """Reusable solver state: workspace and the device info record."""

    def __init__(self, device=None):
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self._ws = {}
        self.barrier_timeout_s = 2.0
        self.inner_tol = 0.1   # reliable-update factor of the mixed-precision solver
        self.max_outer = 60
        self.fft_layout = N.FFT_LAYOUT_AUTO  # spectrum layout of the FFT solves
        # FP32 stencil solves: workspace for double-float residual passes where their error bound allows
        # (False: every reliable update takes an FP64 residual)
        self.df_residual = True

    def workspace(self, n, nrhs, prec, stencil=False):
        """Device workspace of a solve; stencil operators take the size that enables every form."""
        key = (n, nrhs, prec, stencil)
        ws = self._ws.get(key)
        if ws is None:
            query = N.lib().cpm_cg_stencil_workspace_bytes if stencil else N.lib().cpm_cg_workspace_bytes
            nbytes = query(n, nrhs, prec)
            ws = torch.zeros(nbytes, dtype=torch.uint8, device=self.device)
            self._ws[key] = ws
        return ws

    def launch(self, A: DeviceCSR, b: torch.Tensor, x: torch.Tensor, info: torch.Tensor, *, tol, maxiter,
               use_init=False, use_init_dev: torch.Tensor = None, precision="DP", inner_tol=None, form=0,
               precond=None, carry=None):
        """Asynchronous solve; x is read as x0 when use_init, and overwritten.

        form (FP32 stencil solves): N.CG_FORM_DEFAULT (three grid barriers per iteration),
        N.CG_FORM_THREE_BARRIER or N.CG_FORM_TWO_BARRIER (opt-in).
        precond="fft" (FP32 form on a stencil operator with one right-hand side): FP64 refinement
        whose steps solve with the operator's circulant inverse, exactly (one FFT solve per step)
        where the operator pins one node, else as the preconditioner of FP32 CG (inner_tol: the
        residual drop of each inner solve; form=N.CG_FORM_FFT_PCG asks for that form); the plain
        FP32 form is used where the grid has no FFT plan.  carry (a ResidualCarry of the system's size):
        the direct FFT solve keeps its last FP64 residual there, and a warm start from that solve's x
        takes its first residual from it instead of a product (other solves ignore it)."""
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        if precond == "fft" and prec == 1 and hasattr(A, "fft_plan") and b.dim() == 1 and A.fft_plan() is not None:
            return self._launch_fft(A, b, x, info, tol=tol, maxiter=maxiter, use_init=use_init,
                                    use_init_dev=use_init_dev, inner_tol=inner_tol, form=form, carry=carry)
        if prec == 1:
            A.ensure_fp32()
        n = A.shape[0]
        nrhs = 1 if b.dim() == 1 else b.shape[1]
        if b.shape[0] != n or x.shape != b.shape:
            raise ValueError(f"solve shapes: A {A.shape}, b {tuple(b.shape)}, x {tuple(x.shape)}")
        if not (b.is_contiguous() and x.is_contiguous()) or b.dtype != torch.float64 or x.dtype != torch.float64:
            raise TypeError("b and x must be contiguous float64 device tensors")
        stencil = hasattr(A, "ncomp")
        ws = self.workspace(n, nrhs, prec, stencil=stencil and self.df_residual)
        o = N.CGOpts()
        o.tol = float(tol)
        o.maxiter = int(maxiter)
        o.use_init_host = 1 if use_init else 0
        o.use_init_dev = use_init_dev.data_ptr() if use_init_dev is not None else None
        o.precision = prec
        o.inner_tol = self.inner_tol if inner_tol is None else float(inner_tol)
        o.max_outer = self.max_outer
        o.form = int(form)
        o.barrier_timeout_s = self.barrier_timeout_s
        fn = N.lib().cpm_cg_solve_stencil if stencil else N.lib().cpm_cg_solve
        N.check(fn(A.struct(), b.data_ptr(), x.data_ptr(), nrhs, C.byref(o), ws.data_ptr(), ws.numel(),
                   info.data_ptr(), N.stream_ptr()), "cpm_cg_solve")


    def _launch_fft(self, A, b, x, info, *, tol, maxiter, use_init, use_init_dev, inner_tol, form=0, carry=None):
        if b.shape[0] != A.shape[0] or x.shape != b.shape or b.dtype != torch.float64 or x.dtype != torch.float64 \
                or not (b.is_contiguous() and x.is_contiguous()):
            raise ValueError("b and x must be contiguous float64 device vectors of the operator's size")
        key = ("fft", A.nx, A.ny, A.nz, A.ncomp)
        ws = self._ws.get(key)
        if ws is None:
            nbytes = N.lib().cpm_cg_fft_workspace_bytes(A.nx, A.ny, A.nz, A.ncomp)
            ws = torch.zeros(nbytes, dtype=torch.uint8, device=self.device)
            self._ws[key] = ws
        o = N.CGOpts()
        o.tol = float(tol)
        o.maxiter = int(maxiter)
        o.use_init_host = 1 if use_init else 0
        o.use_init_dev = use_init_dev.data_ptr() if use_init_dev is not None else None
        o.precision = 1
        o.inner_tol = 1e-4 if inner_tol is None else float(inner_tol)
        o.form = int(form)
        o.barrier_timeout_s = self.barrier_timeout_s
        if carry is not None:
            if carry.b.shape[0] != b.shape[0] or carry.b.device != b.device:
                raise ValueError("the residual carry must match the system's size and device")
            o.carry_b, o.carry_t, o.carry_valid = carry.b.data_ptr(), carry.t.data_ptr(), carry.valid.data_ptr()
        N.check(N.lib().cpm_cg_solve_stencil_fft(A.struct(), A.fft_plan(self.fft_layout), b.data_ptr(),
                                                 x.data_ptr(), C.byref(o),
                                                 ws.data_ptr(), ws.numel(), info.data_ptr(), N.stream_ptr()),
                "cpm_cg_solve_stencil_fft")


class ResidualCarry:
    """Device storage of the direct FFT solve's residual carry for one system of n unknowns: the b and
    the FP64 residual t = b - A x of its last residual pass, and a flag (int32) that the solve sets when
    x is still the x of that pass.  invalidate() after any change of x other than by the solve."""

    def __init__(self, n, device=None):
        f64 = dict(dtype=torch.float64, device=device or "cuda")
        self.b = torch.zeros(int(n), **f64)
        self.t = torch.zeros(int(n), **f64)
        self.valid = torch.zeros(1, dtype=torch.int32, device=self.b.device)

    def invalidate(self):
        self.valid.zero_()


def new_info(count=1, device=None) -> torch.Tensor:
    """Device storage for `count` cpm_cg_info records."""
    return torch.zeros((count, N.CG_INFO_BYTES), dtype=torch.uint8, device=device or "cuda")


def decode_info(raw: np.ndarray) -> dict:
    b = np.ascontiguousarray(raw).tobytes()
    inf = N.CGInfo.from_buffer_copy(b)
    return {"status": int(inf.status), "iters": list(inf.iters), "outer": int(inf.outer),
            "df_updates": int(inf.df_updates), "resid": list(inf.resid), "bnorm": list(inf.bnorm)}


_default = None


def default_solver() -> CGSolver:
    global _default
    if _default is None:
        N.require_cuda()
        _default = CGSolver()
    return _default


def raise_for(info: dict, A, b, x, system=None, nrhs=1):
    st = info["status"]
    if st == N.CPM_OK:
        return
    if st == N.CPM_NOT_CONVERGED:
        r = b - A.spmv(x)
        rnorm = float(torch.linalg.norm(r))
        its = info["iters"][0] if nrhs == 1 else info["iters"][:nrhs]
        if system is not None:
            msg = f"Error! CG for {system} did not converge. info={its}, residual={rnorm}."
        else:
            msg = f"Error! CG did not converge. info={its}, residual={rnorm}."
        raise RuntimeError(msg)
    raise RuntimeError(f"CG for {system or 'system'} failed: {N.STATUS_NAMES.get(st, st)}")


def solve_cg(A, b, M=None, x0=None, tol=1e-7, maxiter=5000, use_init=False, system=None, precision="DP"):
    """Solve A x = b (A: DeviceCSR or SciPy CSR, b: tensor or array); returns a float64 CUDA tensor.

    Same contract as cupymag/solvers/linear_solvers.py:20-74.  b may hold 3
    right-hand sides as an (n,3) array; they are solved together, each with
    its own stopping test.
    """
    if M is not None:
        raise NotImplementedError("preconditioned CG is not part of the reference path (M must be None)")
    solver = default_solver()
    if not (isinstance(A, DeviceCSR) or hasattr(A, "ncomp")):
        A = DeviceCSR.from_scipy(A)
    b = torch.as_tensor(b, dtype=torch.float64, device=A.device).contiguous()
    if use_init and x0 is not None:
        x = torch.as_tensor(x0, dtype=torch.float64, device=A.device).clone().contiguous()
    else:
        x = torch.zeros_like(b)
    info = new_info(1, A.device)
    solver.launch(A, b, x, info[0], tol=tol, maxiter=maxiter, use_init=bool(use_init and x0 is not None),
                  precision=precision)
    d = decode_info(info[0].cpu().numpy())
    raise_for(d, A, b, x, system=system, nrhs=1 if b.dim() == 1 else b.shape[1])
    return x
