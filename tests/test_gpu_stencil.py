"""Matrix-free hex operators against their CSR form, and the LLG step on them."""
import numpy as np
import pytest
import torch

from . import _golden as G

pytestmark = pytest.mark.gpu


def _sim(case="hex_me_rot", **kw):
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    p = G.params(G.load(case))
    if kw:
        p = p.with_(**kw)
    return SimulationOperators(p), p


@pytest.mark.parametrize("dims", [(6, 6, 6), (7, 5, 9), (6, 5, 8), (4, 4, 4)])
def test_stencil_apply_matches_csr(dims):
    S, p = _sim(Nx=dims[0], Ny=dims[1], Nz=dims[2], Ndx=2, Ndy=2, Ndz=3)
    so = S.stencil_operators()
    csr = S.host_operators()
    rng = np.random.default_rng(3)
    for name, op in so.items():
        A = csr[name]
        x = rng.normal(size=A.shape[1])
        y = op.spmv(torch.as_tensor(x, device="cuda")).cpu().numpy()
        ref = A @ x
        np.testing.assert_allclose(y, ref, rtol=0, atol=1e-13 * np.abs(ref).max(), err_msg=name)
        if op.ncomp == 1:
            X = rng.normal(size=(A.shape[1], 3))
            Y = op.spmv(torch.as_tensor(X, device="cuda")).cpu().numpy()
            np.testing.assert_allclose(Y, A @ X, rtol=0, atol=1e-13 * np.abs(A @ X).max(), err_msg=name)


@pytest.mark.parametrize("dims", [(8, 8, 8), (6, 5, 12)])
def test_quad_product_is_bitwise_the_per_dof_product(dims):
    """nz % 4 == 0 with aligned vectors runs the 4-DOF blocked product; an offset view runs the per-DOF one."""
    S, p = _sim(Nx=dims[0], Ny=dims[1], Nz=dims[2], Ndx=2, Ndy=2, Ndz=2)
    rng = np.random.default_rng(9)
    for name, op in S.stencil_operators().items():
        for nvec in ((1, 3) if op.ncomp == 1 else (1,)):
            shape = (op.shape[1],) if nvec == 1 else (op.shape[1], nvec)
            x = torch.as_tensor(rng.normal(size=shape), device="cuda")
            ya = op.spmv(x)
            buf = torch.empty(x.numel() + 1, dtype=torch.float64, device="cuda")
            xv = buf[1:].view(shape)
            xv.copy_(x)
            ybuf = torch.empty_like(buf)
            yv = ybuf[1:].view(shape)
            op.spmv(xv, out=yv)
            assert torch.equal(ya, yv), (name, nvec)


@pytest.mark.parametrize("dims", [(8, 8, 8), (6, 5, 12), (7, 5, 9), (5, 6, 11), (6, 7, 5), (9, 4, 3)])
def test_fp32_quad_forms_are_bitwise_the_per_dof_product(dims):
    """The FP32 product of the refinement form: scalar-load quads (any nz, quads that cross a z-line end or
    the end of the grid go per DOF) and, for nz % 4 == 0, aligned quads give the per-DOF bits; all three
    agree with the FP64 product to FP32 rounding."""
    S, p = _sim(Nx=dims[0], Ny=dims[1], Nz=dims[2], Ndx=2, Ndy=2, Ndz=2)
    rng = np.random.default_rng(11)
    for name, op in S.stencil_operators().items():
        for nvec in ((1, 3) if op.ncomp == 1 else (1,)):
            shape = (op.shape[1],) if nvec == 1 else (op.shape[1], nvec)
            x64 = torch.as_tensor(rng.normal(size=shape), device="cuda")
            x = x64.float()
            y0 = op.spmv32(x, form=0)
            y2 = op.spmv32(x, form=2)
            assert torch.equal(y0, y2), (name, nvec, dims)
            if dims[2] % 4 == 0:
                assert torch.equal(y0, op.spmv32(x, form=1)), (name, nvec, dims)
            ref = op.spmv(x.double())
            scale = float(ref.abs().max())
            assert float((y0.double() - ref).abs().max()) <= 1e-4 * scale, (name, nvec, dims)


@pytest.mark.parametrize("edge", [12, 11])
@pytest.mark.parametrize("prec", ["DP", "IR"])
def test_stencil_cg_converges_like_csr(prec, edge):
    from cupymag_gb300.solvers.linear_solvers import CGSolver, decode_info, new_info
    S, p = _sim(Nx=edge, Ny=edge, Nz=edge, Ndx=3, Ndy=3, Ndz=3)
    so = S.stencil_operators()
    csr = S.host_operators()
    rng = np.random.default_rng(4)
    for name in ("A_demag", "A1", "A_el"):
        A = csr[name]
        b = rng.normal(size=A.shape[0])
        if name == "A_demag":
            b[0] = 0.0
        if name == "A_el":
            n = A.shape[0] // 3
            b[[0, n, 2 * n]] = 0.0
        bd = torch.as_tensor(b, device="cuda")
        x = torch.zeros_like(bd)
        info = new_info(1)
        CGSolver().launch(so[name], bd, x, info[0], tol=1e-10, maxiter=20000, precision=prec)
        inf = decode_info(info[0].cpu().numpy())
        assert inf["status"] == 0, (name, inf)
        xs = x.cpu().numpy()
        assert np.linalg.norm(b - A @ xs) <= 1e-10 * np.linalg.norm(b) * 1.001, name


@pytest.mark.parametrize("nrhs", [1, 3])
def test_fp32_cg_solves_pinned_dofs_exactly_from_any_start(nrhs):
    """The FP32 refinement CG on A1, whose defect DOFs are pinned (identity rows, excluded columns),
    with b != 0 at those DOFs and a warm start that is wrong there: they come out as x = b exactly
    (the solution of those rows) and the FP64 stopping test holds for every right-hand side."""
    from cupymag_gb300.solvers.linear_solvers import CGSolver, decode_info, new_info
    S, p = _sim(Nx=16, Ny=16, Nz=16, Ndx=5, Ndy=5, Ndz=5)
    op = S.stencil_operators()["A1"]
    A = S.host_operators()["A1"]
    n = A.shape[0]
    rng = np.random.default_rng(8)
    shape = (n, nrhs) if nrhs > 1 else (n,)
    b = rng.normal(size=shape)
    x0 = rng.normal(size=shape)
    bd = torch.as_tensor(b, device="cuda").contiguous()
    x = torch.as_tensor(x0, device="cuda").contiguous()
    info = new_info(1)
    CGSolver().launch(op, bd, x, info[0], tol=1e-10, maxiter=20000, precision="IR", use_init=True)
    inf = decode_info(info[0].cpu().numpy())
    assert inf["status"] == 0, inf
    xs = x.cpu().numpy()
    assert len(S.DefDOF) > 0 and np.array_equal(xs[S.DefDOF], b[S.DefDOF])
    bb, xx = b.reshape(n, -1), xs.reshape(n, -1)
    for r in range(nrhs):
        assert np.linalg.norm(bb[:, r] - A @ xx[:, r]) <= 1e-10 * np.linalg.norm(bb[:, r]) * 1.001, r


@pytest.mark.parametrize("case", ["hex_plain", "hex_me_rot", "hex_me_norot"])
def test_llg_step_on_stencils_matches_reference(case):
    from cupymag_gb300.physics.llg import LLGSolver
    g = G.load(case)
    p = G.params(g)
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    S = SimulationOperators(p)
    L = LLGSolver(S, p, operators="stencil")
    m0 = g["m0"].copy()
    m0[g["DefDOF"]] = 0.0
    L.set_magnetization(torch.as_tensor(m0))
    for k in range(g["step_m"].shape[0]):
        L.step(p.Hext)
        L.check()
        err = np.abs(L.m.cpu().numpy() - g["step_m"][k]).max()
        assert err <= 1e-10, (k, err)


def test_llg_mixed_precision_on_stencils_error_bound():
    from cupymag_gb300.physics.llg import LLGSolver
    from cupymag_gb300.utils.magnetization_io import seeded_initial_m
    S, p = _sim(Nx=16, Ny=16, Nz=16, Ndx=4, Ndy=4, Ndz=4)
    m0 = torch.as_tensor(seeded_initial_m(S.n_dof, S.DefDOF, seed=8))
    A = LLGSolver(S, p, precision="DP")
    B = LLGSolver(S, p, precision="IR", operators="stencil")
    A.set_magnetization(m0)
    B.set_magnetization(m0)
    for _ in range(5):
        A.step(p.Hext)
        B.step(p.Hext)
        A.check()
        B.check()
    assert (A.m - B.m).abs().max().item() <= 1e-6
    assert ((A.avg_m - B.avg_m).abs().max() / A.avg_m.abs().max()).item() <= 1e-6


@pytest.mark.parametrize("edge", [16, 15])
def test_two_barrier_fp32_cg_reaches_the_fp64_stopping_test(edge):
    """The opt-in two-barrier FP32 iteration (s ~ A p carried beside p, one reduction of r.r, r.w, r.s, r.p
    per iteration) reaches the same FP64 stopping test as the default three-barrier form on small grids,
    in at most 1.5x its iterations (GB300, edge 16: demag 67 vs 68, A1 and A2 equal, elasticity 443 vs
    389).  At 128^3 its FP32 recurrences drift and the elastic and demag solves stall, which is why it is
    not the default.  edge 15 runs the per-DOF product, edge 16 the quads."""
    from cupymag_gb300 import _native as N
    from cupymag_gb300.solvers.linear_solvers import CGSolver, decode_info, new_info
    S, p = _sim(Nx=edge, Ny=edge, Nz=edge, Ndx=4, Ndy=4, Ndz=4)
    so = S.stencil_operators()
    csr = S.host_operators()
    rng = np.random.default_rng(12)
    for name, nrhs, inner in (("A_demag", 1, 1e-3), ("A1", 3, 1e-4), ("A1", 1, 1e-4), ("A2", 3, 1e-4),
                              ("A_el", 1, 0.1)):
        A = csr[name]
        b = rng.normal(size=(A.shape[0], nrhs)) if nrhs == 3 else rng.normal(size=A.shape[0])
        if name == "A_demag":
            b[0] = 0.0
        if name == "A_el":
            n = A.shape[0] // 3
            b[[0, n, 2 * n]] = 0.0
        bd = torch.as_tensor(b, device="cuda").contiguous()
        its = {}
        for form in (N.CG_FORM_DEFAULT, N.CG_FORM_TWO_BARRIER):
            x = torch.zeros_like(bd)
            info = new_info(1)
            CGSolver().launch(so[name], bd, x, info[0], tol=1e-10, maxiter=20000, precision="IR", inner_tol=inner,
                              form=form)
            inf = decode_info(info[0].cpu().numpy())
            assert inf["status"] == 0, (name, form, inf)
            xs = x.cpu().numpy()
            res = np.linalg.norm(b - A @ xs, axis=0)
            assert np.all(res <= 1e-10 * np.linalg.norm(b, axis=0) * 1.001), (name, form, res)
            its[form] = inf["iters"][:nrhs]
        print(name, nrhs, "three-barrier", its[0], "two-barrier", its[2])
        for a, c in zip(its[0], its[2]):
            assert c <= 1.5 * a + 3, (name, nrhs, its)


@pytest.mark.parametrize("dims", [(6, 6, 6), (7, 5, 9), (4, 4, 4), (12, 10, 8)])
@pytest.mark.parametrize("rot", [False, True])
def test_matrix_free_derivatives_and_coupling_match_csr(dims, rot):
    """Hd = -F U, the demag right-hand side (shifted by <m>, pinned at DOF 0), the strain from u (with and
    without the [111] rotation) and b_el = F_el E0 (anchor rows empty), matrix-free against the CSR
    matrices of the same grid, to 1e-13 of the largest value."""
    from oracle.llg import R_matrix, strain_from_u
    S, p = _sim(Nx=dims[0], Ny=dims[1], Nz=dims[2], Ndx=2, Ndy=2, Ndz=1, ME=True, rot111=rot)
    D = S.stencil_derivatives()
    F = S.stencil_coupling()
    h = S.host_operators()
    n = S.n_dof
    rng = np.random.default_rng(sum(dims) + rot)
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731

    def close(got, ref, what):
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * np.abs(ref).max(), err_msg=what)

    U = rng.normal(size=n)
    Hd = D.hd_into(dev(U), torch.empty((n, 3), dtype=torch.float64, device="cuda")).cpu().numpy()
    close(Hd, -np.stack([h["Fx"] @ U, h["Fy"] @ U, h["Fz"] @ U], axis=1), "Hd")
    m = rng.normal(size=(n, 3))
    avg = rng.normal(size=3)
    b = D.demag_rhs_into(dev(m), dev(avg), torch.empty(n, dtype=torch.float64, device="cuda"), pin=0).cpu().numpy()
    mt = m - avg
    ref = -(h["Fx"] @ mt[:, 0] + h["Fy"] @ mt[:, 1] + h["Fz"] @ mt[:, 2])
    ref[0] = 0.0
    close(b, ref, "demag rhs")
    u = rng.normal(size=3 * n)
    R = R_matrix() if rot else None
    E = D.compute_E_from_u(n, dev(u), None if R is None else dev(R)).cpu().numpy()
    close(E, strain_from_u(h, n, u, R), "strain")
    E0 = rng.normal(size=6 * n)
    close(F.spmv(dev(E0)).cpu().numpy(), h["F_el"] @ E0, "F_el E0")


@pytest.mark.parametrize("dims", [(16, 16, 16), (15, 13, 11)])
@pytest.mark.parametrize("nrhs", [1, 3])
def test_double_float_residuals_keep_the_fp64_stopping_test(dims, nrhs):
    """FP32 refinement CG whose reliable updates take double-float residuals (A1, A2: scalar, even
    along every axis, symbol bounded away from zero, every flagged row pinned) against the same solves
    with FP64 residuals only: both meet ||b - A x|| <= tol ||b|| on the host in FP64, cold and warm,
    with the same iteration counts to within two, and the double-float solves report their
    double-float updates.  The demag operator (symbol zero at the zero wave vector) takes none and
    gives the same bits either way.  Grids with nz % 4 == 0 run the quad product, the others the
    per-DOF one."""
    from cupymag_gb300.solvers.linear_solvers import CGSolver, decode_info, new_info
    S, p = _sim(Nx=dims[0], Ny=dims[1], Nz=dims[2], Ndx=5, Ndy=5, Ndz=5)
    so = S.stencil_operators()
    csr = S.host_operators()
    rng = np.random.default_rng(21)
    for name in ("A1", "A2", "A_demag"):
        A, op = csr[name], so[name]
        n = A.shape[0]
        shape = (n, nrhs) if nrhs > 1 else (n,)
        b = rng.normal(size=shape)
        if name == "A_demag":
            b.reshape(n, -1)[0] = 0.0
        bd = torch.as_tensor(b, device="cuda").contiguous()
        kick = torch.as_tensor(1e-4 * rng.standard_normal(shape), device="cuda")
        res = {}
        for df in (True, False):
            solver = CGSolver()
            solver.df_residual = df
            x = torch.zeros_like(bd)
            info = new_info(1)
            runs = []
            for warm in (False, True):
                if warm:
                    x += kick
                    x.reshape(n, -1)[S.DefDOF] = 0.0
                solver.launch(op, bd, x, info[0], tol=1e-10, maxiter=20000, precision="IR", use_init=warm)
                inf = decode_info(info[0].cpu().numpy())
                assert inf["status"] == 0, (name, df, warm, inf)
                xs, bb = x.cpu().numpy().reshape(n, -1), b.reshape(n, -1)
                for r in range(nrhs):
                    assert np.linalg.norm(bb[:, r] - A @ xs[:, r]) <= 1e-10 * np.linalg.norm(bb[:, r]), \
                        (name, df, warm, r)
                runs.append((inf, xs.copy()))
            res[df] = runs
        for (idf, xdf), (i64, x64) in zip(res[True], res[False]):
            assert all(abs(a - c) <= 2 for a, c in zip(idf["iters"][:nrhs], i64["iters"][:nrhs])), (name, idf, i64)
            assert i64["df_updates"] == 0
            if name == "A_demag":
                assert idf["df_updates"] == 0 and np.array_equal(xdf, x64), name
            else:
                assert idf["df_updates"] >= 1, (name, idf)
