"""Failure paths of the solvers and the serving loop, made on the host without faulting the GPU.

The reference's only failure mechanism is the RuntimeError of solve_cg when
CuPy's cg reports info != 0 (cupymag/solvers/linear_solvers.py:64-74); that
one is tested with the solver tests.  The kernels here add two statuses:

* CPM_BARRIER_TIMEOUT: every grid-barrier wait is bounded by a launch
  parameter (barrier_timeout_s).  A tiny limit makes the first wait that
  lasts longer than it run out; the kernel then records the status and every
  CTA leaves, so the context stays usable and the next solve on the same
  stream succeeds.
* CPM_NONFINITE: a NaN in the right-hand side makes the CG scalars
  non-finite; the solve stops with that status (in a batch only the system
  that holds the NaN stops).

The serving loop retires a run whose solve failed with its error, and the
other runs of the batch finish with the results they have alone.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

# (operator form, precision): CSR (unstructured path) and matrix-free stencil, FP64 and FP32 + FP64 updates
FORMS = [("csr", "DP"), ("csr", "IR"), ("stencil", "DP"), ("stencil", "IR")]


def _demag(edge=24, form="stencil"):
    """The pinned demag operator of a hex grid and a right-hand side of the demag solve's kind."""
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    from cupymag_gb300.workloads import hex_params
    p = hex_params(edge, edge // 4, False, False)
    S = SimulationOperators(p)
    A = S.stencil_operators()["A_demag"] if form == "stencil" else S.csr_demag_and_deriv()[0]
    rng = np.random.default_rng(edge)
    b = torch.as_tensor(rng.normal(size=S.n_dof), device="cuda")
    b[0] = 0.0
    return A, b


def _solve(solver, A, b, prec):
    from cupymag_gb300.solvers.linear_solvers import decode_info, new_info
    x = torch.zeros_like(b)
    info = new_info(1)
    solver.launch(A, b, x, info[0], tol=1e-10, maxiter=20000, precision=prec)
    torch.cuda.synchronize()
    return x, decode_info(info[0].cpu().numpy())


@pytest.mark.parametrize("form,prec", FORMS)
def test_barrier_timeout_is_reported_and_the_context_stays_usable(form, prec):
    from cupymag_gb300 import _native as N
    from cupymag_gb300.solvers.linear_solvers import CGSolver
    # 48^3: over a hundred CTAs and iterations, so some barrier wait lasts past the first clock reads
    A, b = _demag(edge=48, form=form)
    ref, inf_ref = _solve(CGSolver(), A, b, prec)
    assert inf_ref["status"] == N.CPM_OK
    s = CGSolver()
    s.barrier_timeout_s = 1e-9       # every barrier wait longer than the timer's resolution runs out
    _, inf = _solve(s, A, b, prec)
    assert inf["status"] == N.CPM_BARRIER_TIMEOUT, inf
    # the same solver object, the same stream, the default limit: the solve runs normally
    s.barrier_timeout_s = 2.0
    x, inf2 = _solve(s, A, b, prec)
    assert inf2["status"] == N.CPM_OK
    assert inf2["iters"] == inf_ref["iters"]
    assert torch.equal(x, ref)


@pytest.mark.parametrize("form,prec", FORMS)
def test_nan_right_hand_side_is_reported(form, prec):
    from cupymag_gb300 import _native as N
    from cupymag_gb300.solvers.linear_solvers import CGSolver, raise_for
    A, b = _demag(edge=12, form=form)
    b[77] = float("nan")
    x, inf = _solve(CGSolver(), A, b, prec)
    assert inf["status"] == N.CPM_NONFINITE, inf
    with pytest.raises(RuntimeError, match="non-finite"):
        raise_for(inf, A, b, x, system="demag")


@pytest.mark.parametrize("prec", ["DP", "IR"])
def test_nan_in_one_system_of_a_batch_stops_that_system_only(prec):
    from cupymag_gb300 import _native as N
    from .test_gpu_blockdiag import _solve as bsolve
    from .test_gpu_blockdiag import _systems
    sys_ = _systems(("A_el", 1), [8, 10, 12], prec, seed=9)
    systems = [s for s, _, _ in sys_]
    alone = [bsolve([s], prec)[0] for s in systems]
    systems[1].b[5] = float("nan")
    mix = bsolve(systems, prec)
    assert mix[1][1]["status"] == N.CPM_NONFINITE, mix[1][1]
    for i in (0, 2):
        assert mix[i][1]["status"] == N.CPM_OK
        assert mix[i][1]["iters"] == alone[i][1]["iters"]
        assert np.array_equal(mix[i][0], alone[i][0])


def test_serving_retires_a_failing_run_and_finishes_the_others():
    from cupymag_gb300.serving import Request, ServingEngine

    class NaNRequest(Request):
        """A request whose initial magnetisation carries a NaN (an input error made on the host)."""

        def initial_m(self, n_dof, defect_dofs):
            m = super().initial_m(n_dof, defect_dofs)
            m[n_dof // 2, 1] = float("nan")
            return m

    good = [Request(0, 8, 2, True, 0.12, 5, 11), Request(1, 10, 0, False, 0.07, 4, 12),
            Request(3, 9, 2, True, 0.05, 3, 15)]
    bad = [NaNRequest(2, 8, 1, True, 0.2, 6, 13), NaNRequest(4, 9, 0, False, 0.1, 4, 16)]
    ref, _ = ServingEngine("IR", keep_m=True).serve(good, realtime=False)
    res, st = ServingEngine("IR", keep_m=True).serve(good + bad, realtime=False)
    assert st.failed == len(bad)
    for r in bad:
        assert res[r.rid].error is not None and "non-finite" in res[r.rid].error, res[r.rid].error
        assert res[r.rid].steps < r.steps
    for r in good:
        a, b = ref[r.rid], res[r.rid]
        assert b.error is None and b.steps == r.steps
        assert np.array_equal(a.m, b.m) and np.array_equal(a.hist, b.hist), r.rid
