"""The CG entry point that allocates nothing, against the workspace entry point.

Some callers of this library cannot allocate GPU memory: a host application
that owns every device allocation through its own arena, or an embedding that
forbids cudaMalloc once it has started.  For them cpm_cg_solve_noalloc takes no
workspace and keeps its scratch in a fixed array built into the library.  This
test calls it through the C-ABI twice in a row (one and three right-hand
sides; the second call finds the first call's data in the shared array) and
checks each result against cpm_cg_solve on the same inputs, with the same
tolerance the other solver tests use for identical arithmetic (exact
equality, plus equal iteration counts), in plain FP64 and in the FP32 form
with FP64 refinement (whose five float vectors take the array's larger limit).  It also checks that a solve larger
than the built-in array is refused with an error instead of running.

This file is collected last so that a failure here cannot hide other tests.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from . import _golden as G

pytestmark = pytest.mark.gpu


def _opts(precision=0, tol=1e-10, maxiter=5000):
    from cupymag_gb300 import _native as N
    o = N.CGOpts()
    o.tol, o.maxiter, o.use_init_host, o.use_init_dev = tol, maxiter, 0, None
    o.precision, o.inner_tol, o.max_outer, o.barrier_timeout_s = precision, 1e-5, 60, 2.0
    return o


def _solve_ws(A, b, precision):
    from cupymag_gb300 import _native as N
    from cupymag_gb300.solvers.linear_solvers import decode_info
    nrhs = 1 if b.dim() == 1 else b.shape[1]
    x = torch.zeros_like(b)
    ws = torch.zeros(N.lib().cpm_cg_workspace_bytes(A.shape[0], nrhs, precision), dtype=torch.uint8, device="cuda")
    info = torch.zeros(N.CG_INFO_BYTES, dtype=torch.uint8, device="cuda")
    N.check(N.lib().cpm_cg_solve(A.struct(), b.data_ptr(), x.data_ptr(), nrhs, C.byref(_opts(precision)), ws.data_ptr(),
                                 ws.numel(), info.data_ptr(), N.stream_ptr()), "cpm_cg_solve")
    return x, decode_info(info.cpu().numpy())


def _solve_noalloc(A, b, precision):
    from cupymag_gb300 import _native as N
    from cupymag_gb300.solvers.linear_solvers import decode_info
    nrhs = 1 if b.dim() == 1 else b.shape[1]
    x = torch.zeros_like(b)
    info = torch.zeros(N.CG_INFO_BYTES, dtype=torch.uint8, device="cuda")
    N.check(N.lib().cpm_cg_solve_noalloc(A.struct(), b.data_ptr(), x.data_ptr(), nrhs, C.byref(_opts(precision)),
                                         info.data_ptr(), N.stream_ptr()), "cpm_cg_solve_noalloc")
    return x, decode_info(info.cpu().numpy())


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_cg_matches_workspace_cg_twice(precision):
    from cupymag_gb300 import _native as N
    from cupymag_gb300.utils.device_csr import DeviceCSR
    N.load()
    g = G.load("hex_me_rot")
    rng = np.random.default_rng(21)
    A1 = DeviceCSR.from_scipy(G.matrix(g, "A1"))
    Ad = DeviceCSR.from_scipy(G.matrix(g, "A_demag"))
    b1 = torch.as_tensor(rng.normal(size=Ad.shape[0]), device="cuda")
    b1[0] = 0.0
    b3 = torch.as_tensor(rng.normal(size=(A1.shape[0], 3)), device="cuda")
    if precision == 1:
        A1.ensure_fp32()
        Ad.ensure_fp32()
    for A, b in ((Ad, b1), (A1, b3)):
        x_ref, inf_ref = _solve_ws(A, b, precision)
        x, inf = _solve_noalloc(A, b, precision)
        torch.cuda.synchronize()
        assert inf["status"] == 0 and inf_ref["status"] == 0
        assert inf["iters"] == inf_ref["iters"]
        assert torch.equal(x, x_ref)


def test_noalloc_rejects_oversize_solve():
    from cupymag_gb300 import _native as N
    from cupymag_gb300.utils.device_csr import DeviceCSR
    N.load()
    n = 2_000_000
    # a structurally valid identity matrix larger than the built-in scratch
    ip = torch.arange(n + 1, dtype=torch.int32, device="cuda")
    ix = torch.arange(n, dtype=torch.int32, device="cuda")
    A = DeviceCSR(ip, ix, torch.ones(n, dtype=torch.float64, device="cuda"), (n, n))
    b = torch.ones(n, dtype=torch.float64, device="cuda")
    x = torch.zeros_like(b)
    info = torch.zeros(N.CG_INFO_BYTES, dtype=torch.uint8, device="cuda")
    st = N.lib().cpm_cg_solve_noalloc(A.struct(), b.data_ptr(), x.data_ptr(), 1, C.byref(_opts()), info.data_ptr(),
                                      N.stream_ptr())
    assert st == N.CPM_BAD_ARG
    assert "built-in array" in N.last_error()
