"""Block-diagonal CG plans: many runs' solves in one cooperative launch.

A ``BlockDiagPlan`` is built once per batch composition (it copies the
system table to the device and waits for the copy) and then launched any
number of times, eagerly or inside a captured CUDA graph: the launch reads
tolerances, warm-start flags and vectors through the device pointers it was
built with.  Each system keeps the reference's solve_cg contract
(cupymag/solvers/linear_solvers.py:20-74) and writes its own cpm_cg_info.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from .. import _native as N
from ..solvers.linear_solvers import PRECISIONS


@dataclass
class BlockSystem:
    """One system A x = b of a batch (A: a StencilOperator)."""
    op: object
    b: torch.Tensor
    x: torch.Tensor
    info: torch.Tensor            # (CG_INFO_BYTES,) uint8 device view
    work: torch.Tensor            # uint8 device buffer of at least work_bytes(...)
    tol: float
    maxiter: int
    use_init: torch.Tensor = None  # int32 device flag or None (cold start)

    @property
    def nrhs(self):
        return 1 if self.b.dim() == 1 else int(self.b.shape[1])


def work_bytes(dims, ncomp, nrhs, precision) -> int:
    """Device work bytes of one system on a grid of dims = (nx, ny, nz) cells (cpm_batch_work_bytes)."""
    prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
    nx, ny, nz = (int(v) for v in dims)
    nb = int(N.lib().cpm_batch_work_bytes(nx, ny, nz, int(ncomp), int(nrhs), prec))
    if nb <= 0:
        raise ValueError(f"bad grid {dims} / ncomp {ncomp} / nrhs {nrhs}")
    return nb


def coef_key(op) -> bytes:
    return op.coef_host.tobytes()


class BlockDiagPlan:
    def __init__(self, systems, precision="IR", device=None, inner_tol=0.1, barrier_timeout_s=2.0, form=0):
        if not systems:
            raise ValueError("a block-diagonal plan needs at least one system")
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        op0 = systems[0].op
        ncomp, nrhs, key = op0.ncomp, systems[0].nrhs, coef_key(op0)
        arr = (N.BatchSystem * len(systems))()
        for i, s in enumerate(systems):
            if s.op.ncomp != ncomp or s.nrhs != nrhs or coef_key(s.op) != key:
                raise ValueError("all systems of a plan need the same operator kind and coefficients")
            n = s.op.n * s.op.ncomp
            if s.b.shape[0] != n or s.x.shape != s.b.shape or s.b.dtype != torch.float64 or not s.b.is_contiguous() \
                    or not s.x.is_contiguous():
                raise ValueError(f"system {i}: b, x must be contiguous float64 of {n} rows")
            if s.work.numel() < work_bytes((s.op.nx, s.op.ny, s.op.nz), ncomp, nrhs, self.precision) or \
                    s.work.data_ptr() % 256:
                raise ValueError(f"system {i}: work buffer too small or not 256-byte aligned")
            e = arr[i]
            e.nx, e.ny, e.nz = s.op.nx, s.op.ny, s.op.nz
            e.maxiter, e.tol = int(s.maxiter), float(s.tol)
            e.flags = None if s.op.flags is None else s.op.flags.data_ptr()
            e.b, e.x = s.b.data_ptr(), s.x.data_ptr()
            e.use_init_dev = None if s.use_init is None else s.use_init.data_ptr()
            e.info, e.work = s.info.data_ptr(), s.work.data_ptr()
        L = N.lib()
        nbytes = N.i64()
        N.check(L.cpm_batch_plan_bytes(arr, len(systems), ncomp, nrhs, self.precision, C.byref(nbytes)),
                "cpm_batch_plan_bytes")
        dev = device or systems[0].b.device
        self.mem = torch.empty(int(nbytes.value), dtype=torch.uint8, device=dev)
        if self.mem.data_ptr() % 256:
            raise RuntimeError("plan memory is not 256-byte aligned")
        coef = (C.c_double * 243)()
        coef[:op0.coef_host.size] = tuple(float(v) for v in op0.coef_host)
        self.plan = N.BatchPlan()
        N.check(L.cpm_batch_plan_build(arr, len(systems), ncomp, nrhs, self.precision, coef, self.mem.data_ptr(),
                                       nbytes.value, C.byref(self.plan), N.stream_ptr()), "cpm_batch_plan_build")
        self.opts = N.CGOpts()
        self.opts.inner_tol = float(inner_tol)
        self.opts.barrier_timeout_s = float(barrier_timeout_s)
        self.opts.form = int(form)   # FP32: N.CG_FORM_DEFAULT (three barriers) or N.CG_FORM_TWO_BARRIER
        self.systems = list(systems)   # keeps every buffer the plan points to alive
        self.ncomp, self.nrhs = ncomp, nrhs

    @property
    def grid(self):
        return int(self.plan.grid)

    def launch(self):
        """Solve every system (asynchronous on the current stream; one kernel)."""
        N.check(N.lib().cpm_cg_solve_blockdiag(C.byref(self.plan), C.byref(self.opts), N.stream_ptr()),
                "cpm_cg_solve_blockdiag")
