"""Serving loop: continuous batching, alone-vs-mix identity, budget admission."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _reqs():
    from cupymag_gb300.serving import Request
    return [Request(0, 8, 2, True, 0.12, 6, 11), Request(1, 10, 0, False, 0.07, 4, 12),
            Request(2, 6, 1, True, 0.2, 8, 13), Request(3, 12, 3, False, 0.15, 5, 14),
            Request(4, 9, 2, True, 0.05, 3, 15)]


@pytest.mark.parametrize("prec", ["DP", "IR"])
def test_result_is_the_same_alone_and_in_the_mix(prec):
    from cupymag_gb300.serving import ServingEngine
    reqs = _reqs()
    mix, st = ServingEngine(prec, keep_m=True).serve(reqs, realtime=False)
    assert st.failed == 0 and st.max_batch == len(reqs)
    assert st.graph_error is None and st.graph_steps > 0
    for r in reqs:
        alone, _ = ServingEngine(prec, keep_m=True, use_graphs=(r.rid % 2 == 0)).serve([r], realtime=False)
        a, b = alone[r.rid], mix[r.rid]
        assert a.error is None and b.error is None
        assert a.steps == b.steps == r.steps
        assert np.array_equal(a.m, b.m), (prec, r.rid)
        assert np.array_equal(a.hist, b.hist), (prec, r.rid)


def test_served_runs_match_sequential_fp64():
    from cupymag_gb300.serving import ServingEngine, run_sequential
    reqs = _reqs()
    seq, _ = run_sequential(reqs, precision="DP", keep_m=True)
    dp, _ = ServingEngine("DP", keep_m=True).serve(reqs, realtime=False)
    ir, _ = ServingEngine("IR", keep_m=True).serve(reqs, realtime=False)
    for r in reqs:
        s = seq[r.rid]
        assert s.error is None
        assert np.abs(dp[r.rid].m - s.m).max() <= 1e-10, r.rid
        assert np.abs(dp[r.rid].hist[:, :3] - s.hist[:, :3]).max() <= 1e-10
        assert np.abs(ir[r.rid].m - s.m).max() <= 1e-6, r.rid
        rel = np.abs(ir[r.rid].hist[:, :3] - s.hist[:, :3]).max() / np.abs(s.hist[:, :3]).max()
        assert rel <= 1e-6


def test_sequential_schedule_matches_host_field_steps():
    """The device field schedule gives the same trajectory as passing Hext per step."""
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    from cupymag_gb300.physics.llg import LLGSolver
    from cupymag_gb300.serving import run_sequential
    from cupymag_gb300.workloads import seeded_m0
    r = _reqs()[0]
    seq, _ = run_sequential([r], keep_m=True)
    p = r.params()
    S = SimulationOperators(p)
    L = LLGSolver(S, p, precision="DP", operators="stencil")
    L.set_magnetization(torch.as_tensor(seeded_m0(S.n_dof, S.DefDOF, r.seed)))
    for H in r.fields(p):
        L.step(H)
        L.check()
    assert np.array_equal(L.m.cpu().numpy(), seq[r.rid].m)


def test_budget_admission_serialises_runs():
    from cupymag_gb300.serving import ServingEngine, estimate_bytes
    reqs = _reqs()[:3]
    big = max(estimate_bytes(r.params(), "IR") for r in reqs)
    eng = ServingEngine("IR", hbm_budget_gb=1.5 * big / 1e9)
    res, st = eng.serve(reqs, realtime=False)
    assert st.max_batch == 1 and st.failed == 0 and len(res) == 3
    tiny = ServingEngine("IR", hbm_budget_gb=1e-6)
    res, st = tiny.serve(reqs[:1], realtime=False)
    assert res[0].error == "request exceeds the HBM budget"


def test_estimate_covers_allocation():
    from cupymag_gb300.serving import ServingEngine, estimate_bytes
    from cupymag_gb300.serving.workload import Request
    for r in (Request(0, 24, 4, True, 0.1, 1, 1), Request(1, 24, 4, False, 0.1, 1, 2),
              Request(2, 32, 4, True, 0.1, 1, 3), Request(3, 34, 0, False, 0.1, 1, 4)):
        eng = ServingEngine("IR")
        torch.cuda.synchronize()
        before = torch.cuda.memory_allocated()
        eng.admit(r, 0.0)
        eng.step()
        torch.cuda.synchronize()
        used = torch.cuda.memory_allocated() - before
        assert used <= estimate_bytes(r.params(), "IR"), (r.ME, used)


def test_realtime_arrivals_overlap():
    """Requests arriving while others run join the running batch (continuous batching)."""
    from cupymag_gb300.serving import Request, ServingEngine
    reqs = [Request(i, 10 + i, 1, i % 2 == 0, 0.1, 40, 100 + i, arrival=0.01 * i) for i in range(4)]
    res, st = ServingEngine("IR").serve(reqs, realtime=True)
    assert st.failed == 0 and st.max_batch >= 2
    assert all(res[r.rid].steps == r.steps for r in reqs)
    assert st.latency_p99_s >= st.latency_p50_s > 0


def test_operator_cache_shares_operators_of_identical_grids():
    """Runs with the same grid, defect and material share one set of matrix-free operators; their results
    are the ones each has when served by an engine of its own."""
    from cupymag_gb300.serving import Request, ServingEngine
    reqs = [Request(0, 10, 2, True, 0.1, 3, 21), Request(1, 10, 2, True, 0.15, 3, 22),
            Request(2, 10, 2, False, 0.1, 3, 23), Request(3, 10, 2, True, 0.05, 3, 24)]
    eng = ServingEngine("IR", keep_m=True)
    res, st = eng.serve(reqs, realtime=False)
    assert st.failed == 0
    assert eng.cache.misses == 2 and eng.cache.hits == 2
    for r in reqs:
        alone, _ = ServingEngine("IR", keep_m=True).serve([r], realtime=False)
        assert np.array_equal(alone[r.rid].m, res[r.rid].m), r.rid


def test_fft_solved_runs_are_the_same_alone_and_in_the_mix():
    """Runs of 32^3 and up solve elasticity and demag with the FFT-preconditioned solver, one launch per
    run, beside block-diagonal launches for the small runs: every result is the same alone and in the mix
    (bit for bit) and within 1e-6 of the same run in plain FP64."""
    from cupymag_gb300.serving import Request, ServingEngine, run_sequential
    reqs = [Request(0, 32, 4, True, 0.12, 4, 31), Request(1, 10, 2, False, 0.07, 4, 32),
            Request(2, 34, 0, False, 0.1, 3, 33), Request(3, 8, 2, True, 0.2, 5, 34)]
    eng = ServingEngine("IR", keep_m=True)
    mix, st = eng.serve(reqs, realtime=False)
    assert st.failed == 0 and st.fft_launches > 0 and st.graph_steps > 0
    seq, _ = run_sequential(reqs, precision="DP", keep_m=True)
    for r in reqs:
        alone, _ = ServingEngine("IR", keep_m=True).serve([r], realtime=False)
        assert np.array_equal(alone[r.rid].m, mix[r.rid].m), r.rid
        assert np.array_equal(alone[r.rid].hist, mix[r.rid].hist), r.rid
        assert np.abs(mix[r.rid].m - seq[r.rid].m).max() <= 1e-6, r.rid
