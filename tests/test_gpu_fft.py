"""The circulant (FFT) preconditioner and the preconditioned FP32 CG inside FP64 refinement.

The elastic and demag operators of the periodic hex grid are block-circulant
except for the anchor at DOF 0; the preconditioner applies the inverse of the
circulant part (the singular zero wave vector replaced by the operator's
diagonal) with DFTs along each axis in shared memory.  Checked here:

* z = M r against the same inverse computed on the host with numpy's FFT, on
  grids whose line lengths have factors 2, 3, 4, 5, 7, 8, 11 and primes, in
  both spectrum layouts (the half spectrum of x-planes in shared memory, and
  five passes over the full spectrum);
* both FFT solves meet the FP64 stopping test ||b - A x|| <= tol ||b|| (status
  ok) in far fewer iterations than plain FP32 CG, cold and warm, and return b
  for b = 0 (cupyx semantics, cupymag/solvers/linear_solvers.py:59-74): the
  direct refinement (the anchored operator inverted exactly by one FFT solve
  per FP64 step) and FP32 CG preconditioned by the circulant inverse;
* the direct step alone is the exact inverse of the anchored operator: one
  step from x = 0 against the host's dense solve;
* the residual carry of the direct solve (the first residual of a warm start
  taken from the previous solve's FP64 residual) against warm starts without it.
"""
import numpy as np
import pytest
import torch

from . import _golden as G

pytestmark = pytest.mark.gpu


def _sim(**kw):
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    p = G.params(G.load("hex_me_rot")).with_(**kw)
    return SimulationOperators(p), p


def _host_inverse(coef, nc, dims, r):
    """M r on the host: DFT, per-wave-vector solve with the stencil's symbol (zero wave vector: the
    operator's diagonal), inverse DFT."""
    nx, ny, nz = dims
    c = np.asarray(coef, dtype=np.float64).reshape(nc, nc, 3, 3, 3)
    tx, ty, tz = (2 * np.pi * np.arange(m) / m for m in dims)
    S = np.zeros((nx, ny, nz, nc, nc))
    for dx in range(3):
        for dy in range(3):
            for dz in range(3):
                ph = np.cos(tx[:, None, None] * (dx - 1) + ty[None, :, None] * (dy - 1) + tz[None, None, :] * (dz - 1))
                S += ph[..., None, None] * c[:, :, dx, dy, dz]
    S[0, 0, 0] = np.eye(nc) * np.trace(c[:, :, 1, 1, 1]) / nc
    R = np.fft.fftn(r.reshape(nc, nx, ny, nz), axes=(1, 2, 3))
    U = np.einsum("xyzab,bxyz->axyz", np.linalg.inv(S), R)
    return np.fft.ifftn(U, axes=(1, 2, 3)).real.reshape(-1)


LAYOUTS = ["slab", "passes"]


def _layout(name):
    from cupymag_gb300 import _native as N
    return {"slab": N.FFT_LAYOUT_SLAB, "passes": N.FFT_LAYOUT_PASSES}[name]


@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("dims", [(8, 8, 8), (6, 10, 12), (5, 7, 11), (12, 16, 20), (9, 4, 3), (13, 6, 14),
                                  (16, 24, 32)])
def test_fft_preconditioner_is_the_circulant_inverse(dims, layout):
    S, p = _sim(Nx=dims[0], Ny=dims[1], Nz=dims[2], Ndx=1, Ndy=1, Ndz=1, ME=True)
    so = S.stencil_operators()
    rng = np.random.default_rng(sum(dims))
    for name in ("A_demag", "A_el"):
        op = so[name]
        r = rng.normal(size=op.shape[0]).astype(np.float32)
        z = op.precondition32(torch.as_tensor(r, device="cuda"), layout=_layout(layout)).cpu().numpy()
        assert op.fft_plan(_layout(layout)).layout == _layout(layout)
        ref = _host_inverse(op.coef_host, op.ncomp, dims, r.astype(np.float64))
        err = np.abs(z - ref).max() / np.abs(ref).max()
        assert err <= 1e-4, (name, dims, layout, err)


def test_fft_plan_picks_the_slab_layout_where_it_fits():
    from cupymag_gb300 import _native as N
    S, p = _sim(Nx=12, Ny=10, Nz=14, Ndx=3, Ndy=3, Ndz=3, ME=True)
    so = S.stencil_operators()
    for name in ("A_demag", "A_el"):
        assert so[name].fft_plan().layout == N.FFT_LAYOUT_SLAB


METHODS = ["direct", "pcg"]


def _form(method):
    from cupymag_gb300 import _native as N
    return N.CG_FORM_DEFAULT if method == "direct" else N.CG_FORM_FFT_PCG


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("dims", [(16, 16, 16), (15, 15, 15), (12, 10, 14)])
def test_fft_solves_meet_the_fp64_stopping_test(dims, layout, method):
    from cupymag_gb300 import _native as N
    from cupymag_gb300.solvers.linear_solvers import CGSolver, decode_info, new_info
    S, p = _sim(Nx=dims[0], Ny=dims[1], Nz=dims[2], Ndx=3, Ndy=3, Ndz=3, ME=True)
    so = S.stencil_operators()
    csr = S.host_operators()
    rng = np.random.default_rng(7)
    for name in ("A_demag", "A_el"):
        A = csr[name]
        n = A.shape[0] // so[name].ncomp
        b = rng.normal(size=A.shape[0])
        b[[0, n, 2 * n] if name == "A_el" else [0]] = 0.0
        bd = torch.as_tensor(b, device="cuda")
        res = {}
        solver = CGSolver()
        solver.fft_layout = _layout(layout)
        for precond in ("fft", None):
            x = torch.zeros_like(bd)
            info = new_info(1)
            solver.launch(so[name], bd, x, info[0], tol=1e-10, maxiter=20000, precision="IR",
                          inner_tol=1e-4 if precond else 0.1, precond=precond,
                          form=_form(method) if precond else 0)
            inf = decode_info(info[0].cpu().numpy())
            assert inf["status"] == N.CPM_OK, (name, precond, inf)
            xs = x.cpu().numpy()
            assert np.linalg.norm(b - A @ xs) <= 1e-10 * np.linalg.norm(b) * 1.001, (name, precond)
            res[precond] = (inf["iters"][0], xs)
        print(name, dims, layout, method, "FFT", res["fft"][0], "plain", res[None][0])
        assert res["fft"][0] * 3 <= res[None][0], (name, dims, res["fft"][0], res[None][0])
        if method == "direct":
            assert so[name].anchor == 0 and res["fft"][0] <= 4, (name, dims, res["fft"][0])
        # warm start from the solution: converged at the first FP64 residual, no inner iteration
        x = torch.as_tensor(res["fft"][1], device="cuda")
        info = new_info(1)
        solver.launch(so[name], bd, x, info[0], tol=1e-10, maxiter=20000, precision="IR", use_init=True,
                      precond="fft", form=_form(method))
        inf = decode_info(info[0].cpu().numpy())
        assert inf["status"] == N.CPM_OK and inf["iters"][0] == 0, inf
        # zero right-hand side: x = b
        z = torch.zeros_like(bd)
        x = torch.full_like(bd, 3.0)
        solver.launch(so[name], z, x, info[0], tol=1e-10, maxiter=20000, precision="IR", precond="fft",
                      form=_form(method))
        inf = decode_info(info[0].cpu().numpy())
        assert inf["status"] == N.CPM_OK and float(x.abs().max()) == 0.0


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("layout", LAYOUTS)
def test_fft_solve_reports_maxiter_like_the_reference(layout, method):
    from cupymag_gb300 import _native as N
    from cupymag_gb300.solvers.linear_solvers import CGSolver, decode_info, new_info
    S, p = _sim(Nx=12, Ny=12, Nz=12, Ndx=3, Ndy=3, Ndz=3, ME=True)
    op = S.stencil_operators()["A_el"]
    rng = np.random.default_rng(3)
    b = torch.as_tensor(rng.normal(size=op.shape[0]), device="cuda")
    b[[0, op.n, 2 * op.n]] = 0.0
    x = torch.zeros_like(b)
    info = new_info(1)
    solver = CGSolver()
    solver.fft_layout = _layout(layout)
    cap = 1 if method == "direct" else 3
    solver.launch(op, b, x, info[0], tol=1e-10, maxiter=cap, precision="IR", precond="fft", form=_form(method))
    inf = decode_info(info[0].cpu().numpy())
    assert inf["status"] == N.CPM_NOT_CONVERGED and inf["iters"][0] == cap, inf


@pytest.mark.parametrize("layout", LAYOUTS)
@pytest.mark.parametrize("dims", [(6, 7, 8), (9, 4, 5)])
def test_direct_step_is_the_exact_inverse_of_the_anchored_operator(dims, layout):
    """One direct step from x = 0 (maxiter 1) solves A x = b to FP32 accuracy, b with a nonzero
    value at the anchor (the correction terms at its neighbours and at the anchor all act)."""
    from cupymag_gb300.solvers.linear_solvers import CGSolver, new_info
    S, p = _sim(Nx=dims[0], Ny=dims[1], Nz=dims[2], Ndx=1, Ndy=1, Ndz=1, ME=True)
    so = S.stencil_operators()
    csr = S.host_operators()
    rng = np.random.default_rng(5)
    for name in ("A_demag", "A_el"):
        A = csr[name].toarray()
        b = rng.normal(size=A.shape[0])
        ref = np.linalg.solve(A, b)
        x = torch.zeros(A.shape[0], dtype=torch.float64, device="cuda")
        info = new_info(1)
        solver = CGSolver()
        solver.fft_layout = _layout(layout)
        solver.launch(so[name], torch.as_tensor(b, device="cuda"), x, info[0], tol=1e-30, maxiter=1,
                      precision="IR", precond="fft")
        err = np.abs(x.cpu().numpy() - ref).max() / np.abs(ref).max()
        assert err <= 1e-4, (name, dims, layout, err)


@pytest.mark.parametrize("layout", LAYOUTS)
def test_direct_solve_residual_carry(layout):
    """The residual carry of the direct solve: after a solve it holds b and the FP64 residual of the
    returned x (flag 1, also when maxiter stops the solve); warm starts that take their first residual
    from it meet the FP64 stopping test like warm starts without it; a changed x with the flag cleared
    is solved from an FP64 residual; b = 0 and the preconditioned-CG form clear the flag; the C-ABI
    refuses a partial or aliased carry."""
    import types
    from cupymag_gb300 import _native as N
    from cupymag_gb300.solvers.linear_solvers import CGSolver, ResidualCarry, decode_info, new_info
    S, p = _sim(Nx=12, Ny=10, Nz=14, Ndx=3, Ndy=3, Ndz=3, ME=True)
    so = S.stencil_operators()
    csr = S.host_operators()
    rng = np.random.default_rng(11)
    solver = CGSolver()
    solver.fft_layout = _layout(layout)
    eps = np.finfo(np.float64).eps
    for name in ("A_demag", "A_el"):
        A = csr[name]
        n = A.shape[0] // so[name].ncomp
        pins = [0, n, 2 * n] if name == "A_el" else [0]
        b0 = rng.normal(size=A.shape[0])
        b0[pins] = 0.0
        delta = rng.normal(size=A.shape[0])
        delta[pins] = 0.0
        carry = ResidualCarry(A.shape[0])
        info = new_info(1)

        def solve(b, x, use_init, carry=carry, maxiter=20000, form=_form("direct")):
            solver.launch(so[name], torch.as_tensor(b, device="cuda"), x, info[0], tol=1e-10, maxiter=maxiter,
                          precision="IR", use_init=use_init, precond="fft", form=form, carry=carry)
            return decode_info(info[0].cpu().numpy())

        def carry_matches(b, x):
            xs = x.cpu().numpy()
            bound = 64 * eps * (abs(A) @ np.abs(xs) + np.abs(b))
            assert np.array_equal(carry.b.cpu().numpy(), b), name
            assert np.all(np.abs(carry.t.cpu().numpy() - (b - A @ xs)) <= bound), name
            assert int(carry.valid.item()) == 1, name

        # cold solve: the carry holds b and the residual of x
        x = torch.zeros(A.shape[0], dtype=torch.float64, device="cuda")
        inf = solve(b0, x, False)
        assert inf["status"] == N.CPM_OK, inf
        carry_matches(b0, x)
        # warm starts from the carry against warm starts without it
        x_plain = x.clone()
        for k in range(1, 4):
            b = b0 + 1e-3 * k * delta
            inf = solve(b, x, True)
            inf_plain = solve(b, x_plain, True, carry=None)
            for xx, ii in ((x, inf), (x_plain, inf_plain)):
                assert ii["status"] == N.CPM_OK, (name, k, ii)
                assert np.linalg.norm(b - A @ xx.cpu().numpy()) <= 1e-10 * np.linalg.norm(b) * 1.001, (name, k)
            assert abs(inf["iters"][0] - inf_plain["iters"][0]) <= 1, (name, k, inf, inf_plain)
            carry_matches(b, x)
        # the same b again: the carried residual meets the test, an FP64 residual confirms it, no step
        inf = solve(b, x, True)
        assert inf["status"] == N.CPM_OK and inf["iters"][0] == 0, inf
        carry_matches(b, x)
        # x changed by the caller, flag cleared: solved from an FP64 residual
        x += torch.as_tensor(1e-3 * delta, device="cuda")
        carry.invalidate()
        inf = solve(b, x, True)
        assert inf["status"] == N.CPM_OK and inf["iters"][0] >= 1, inf
        assert np.linalg.norm(b - A @ x.cpu().numpy()) <= 1e-10 * np.linalg.norm(b) * 1.001, name
        carry_matches(b, x)
        # stopped by maxiter: the carry still describes the returned x
        x.zero_()
        inf = solve(b0, x, False, maxiter=1)
        assert inf["status"] == N.CPM_NOT_CONVERGED, inf
        carry_matches(b0, x)
        # b = 0 (x = b) and the preconditioned-CG form leave no valid carry
        inf = solve(np.zeros_like(b0), x, True)
        assert inf["status"] == N.CPM_OK and int(carry.valid.item()) == 0, inf
        x.zero_()
        solve(b0, x, False)
        assert int(carry.valid.item()) == 1
        solve(b0, x, True, form=_form("pcg"))
        assert int(carry.valid.item()) == 0
        # a partial carry or one that aliases x is refused before any launch
        bad = types.SimpleNamespace(b=carry.b, t=carry.t, valid=types.SimpleNamespace(data_ptr=lambda: 0))
        with pytest.raises(RuntimeError, match="together"):
            solve(b0, x, True, carry=bad)
        alias = types.SimpleNamespace(b=x, t=carry.t, valid=carry.valid)
        with pytest.raises(RuntimeError, match="alias"):
            solve(b0, x, True, carry=alias)
