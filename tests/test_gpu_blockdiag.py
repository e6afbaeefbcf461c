"""Block-diagonal CG: one launch over systems of different sizes."""
import numpy as np
import pytest
import torch

from . import _golden as G

pytestmark = pytest.mark.gpu


def _ops(edge, defect, ME=True):
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    from cupymag_gb300.workloads import hex_params
    p = hex_params(edge, defect, ME, ME)
    S = SimulationOperators(p)
    return S.stencil_operators(), S.host_operators(), p


def _systems(kind, edges, prec, seed=0, maxiter=20000):
    from cupymag_gb300.serving.blockdiag import BlockSystem, work_bytes
    from cupymag_gb300.solvers.linear_solvers import new_info
    name, nrhs = kind
    rng = np.random.default_rng(seed)
    out = []
    for e in edges:
        so, host, p = _ops(e, max(1, e // 4))
        op, A = so[name], host[name]
        n = A.shape[0]
        b = rng.normal(size=(n, nrhs)) if nrhs == 3 else rng.normal(size=n)
        if name == "A_demag":
            b[0] = 0.0
        if name == "A_el":
            b[[0, n // 3, 2 * n // 3]] = 0.0
        bd = torch.as_tensor(b, device="cuda").contiguous()
        x = torch.zeros_like(bd)
        info = new_info(1)[0]
        work = torch.empty(work_bytes((op.nx, op.ny, op.nz), op.ncomp, nrhs, prec), dtype=torch.uint8, device="cuda")
        out.append((BlockSystem(op, bd, x, info, work, 1e-10, maxiter), A, b))
    return out


def _solve(systems, prec):
    from cupymag_gb300.serving.blockdiag import BlockDiagPlan
    from cupymag_gb300.solvers.linear_solvers import decode_info
    for s in systems:
        s.x.zero_()
    plan = BlockDiagPlan(systems, prec)
    plan.launch()
    torch.cuda.synchronize()
    return [(s.x.cpu().numpy(), decode_info(s.info.cpu().numpy())) for s in systems]


KINDS = [("A_demag", 1), ("A1", 3), ("A_el", 1)]


@pytest.mark.parametrize("prec", ["DP", "IR"])
@pytest.mark.parametrize("kind", KINDS, ids=[k[0] + str(k[1]) for k in KINDS])
def test_blockdiag_alone_equals_in_mix(kind, prec):
    sys_ = _systems(kind, [7, 12, 9, 16], prec)
    mix = _solve([s for s, _, _ in sys_], prec)
    for i, (s, A, b) in enumerate(sys_):
        alone = _solve([s], prec)[0]
        assert np.array_equal(alone[0], mix[i][0]), (kind, prec, i)
        assert alone[1] == mix[i][1]
        inf = mix[i][1]
        assert inf["status"] == 0, inf
        x = mix[i][0]
        r = b - A @ x
        nb = np.linalg.norm(b, axis=0)
        assert np.all(np.linalg.norm(r, axis=0) <= 1e-10 * nb * 1.001), (kind, prec, i)


@pytest.mark.parametrize("prec", ["DP", "IR"])
def test_blockdiag_iterations_match_single_solver(prec):
    from cupymag_gb300.solvers.linear_solvers import CGSolver, decode_info, new_info
    sys_ = _systems(("A_el", 1), [10, 14], prec, seed=3)
    mix = _solve([s for s, _, _ in sys_], prec)
    for (s, A, b), (x, inf) in zip(sys_, mix):
        xs = torch.zeros_like(s.b)
        info = new_info(1)
        CGSolver().launch(s.op, s.b, xs, info[0], tol=1e-10, maxiter=20000, precision=prec)
        d = decode_info(info[0].cpu().numpy())
        slack = 1 if prec == "DP" else max(3, d["iters"][0] // 50)
        assert abs(d["iters"][0] - inf["iters"][0]) <= slack, (d["iters"], inf["iters"])
        if prec == "DP":
            np.testing.assert_allclose(x, xs.cpu().numpy(), rtol=0, atol=1e-8 * np.abs(x).max())


def test_blockdiag_maxiter_is_per_system():
    from cupymag_gb300 import _native as N
    sys_ = _systems(("A_demag", 1), [8, 8], "DP", seed=5)
    sys_[1][0].maxiter = 3
    res = _solve([s for s, _, _ in sys_], "DP")
    assert res[0][1]["status"] == N.CPM_OK
    assert res[1][1]["status"] == N.CPM_NOT_CONVERGED and res[1][1]["iters"][0] == 3


def test_blockdiag_warm_start_and_zero_rhs():
    from cupymag_gb300.serving.blockdiag import BlockDiagPlan
    from cupymag_gb300.solvers.linear_solvers import decode_info
    sys_ = _systems(("A_demag", 1), [8, 9], "DP", seed=6)
    s0, s1 = sys_[0][0], sys_[1][0]
    s1.b.zero_()
    flag = torch.ones(1, dtype=torch.int32, device="cuda")
    s0.use_init = flag
    s1.use_init = flag
    A0 = sys_[0][1]
    x_true = np.linalg.lstsq(A0.toarray(), sys_[0][2], rcond=None)[0] if A0.shape[0] < 800 else None
    s0.x.copy_(torch.as_tensor(x_true, device="cuda"))
    s1.x.fill_(3.0)
    plan = BlockDiagPlan([s0, s1], "DP")
    plan.launch()
    torch.cuda.synchronize()
    d0 = decode_info(s0.info.cpu().numpy())
    d1 = decode_info(s1.info.cpu().numpy())
    assert d0["status"] == 0 and d0["iters"][0] <= 2
    assert d1["status"] == 0 and d1["iters"][0] == 0 and float(s1.x.abs().max()) == 0.0


def test_blockdiag_rejects_mixed_kinds():
    from cupymag_gb300.serving.blockdiag import BlockDiagPlan
    a = _systems(("A_demag", 1), [8], "DP")[0][0]
    b = _systems(("A1", 1), [8], "DP")[0][0]
    with pytest.raises(ValueError):
        BlockDiagPlan([a, b], "DP")


@pytest.mark.parametrize("kind", KINDS, ids=[k[0] + str(k[1]) for k in KINDS])
def test_blockdiag_two_barrier_form_alone_equals_in_mix(kind):
    """The opt-in two-barrier FP32 form of the block-diagonal kernel: each system's iterates are the same
    alone and in a mix (bit for bit), and every system meets the FP64 stopping test."""
    from cupymag_gb300 import _native as N
    from cupymag_gb300.serving.blockdiag import BlockDiagPlan
    from cupymag_gb300.solvers.linear_solvers import decode_info

    def solve(systems):
        for s in systems:
            s.x.zero_()
        BlockDiagPlan(systems, "IR", form=N.CG_FORM_TWO_BARRIER).launch()
        torch.cuda.synchronize()
        return [(s.x.cpu().numpy(), decode_info(s.info.cpu().numpy())) for s in systems]

    sys_ = _systems(kind, [7, 12, 9, 16], "IR", seed=4)
    mix = solve([s for s, _, _ in sys_])
    for i, (s, A, b) in enumerate(sys_):
        alone = solve([s])[0]
        assert np.array_equal(alone[0], mix[i][0]), (kind, i)
        assert alone[1] == mix[i][1]
        assert mix[i][1]["status"] == 0, mix[i][1]
        r = b - A @ mix[i][0]
        assert np.all(np.linalg.norm(r, axis=0) <= 1e-10 * np.linalg.norm(b, axis=0) * 1.001), (kind, i)
