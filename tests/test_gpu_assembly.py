"""Device-side COO assembly for unstructured meshes against the host (SciPy) path."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_segment_sum_is_in_order_and_exact():
    from cupymag_gb300 import _native as N
    rng = np.random.default_rng(0)
    vals = rng.normal(size=1000)
    counts = rng.integers(1, 9, size=200)
    counts[-1] = 1000 - counts[:-1].sum() if counts[:-1].sum() < 1000 else 1
    counts = counts[np.cumsum(counts) <= 1000]
    start = np.concatenate([[0], np.cumsum(counts)])
    v = torch.as_tensor(vals[:start[-1]], device="cuda")
    st = torch.as_tensor(start, dtype=torch.int64, device="cuda")
    out = torch.empty(len(counts), dtype=torch.float64, device="cuda")
    N.check(N.lib().cpm_coo_segment_sum(v.data_ptr(), st.data_ptr(), len(counts), out.data_ptr(),
                                        N.stream_ptr()), "segment sum")
    ref = []
    for a, b in zip(start[:-1], start[1:]):
        acc = 0.0
        for x in vals[a:b]:
            acc += x
        ref.append(acc)
    assert np.array_equal(out.cpu().numpy(), np.array(ref))


@pytest.mark.parametrize("me", [True, False])
def test_device_assembly_matches_host(me):
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    from cupymag_gb300.workloads import tet_workload
    w = dict(n=8, jitter=0.2, axes=(0.3, 0.2, 0.15), ME=me, rot111=me, seed=5)
    p, mesh = tet_workload(w)
    H = SimulationOperators(p, assembly="coo", mesh=mesh).host_operators()
    D = SimulationOperators(p, assembly="device", mesh=mesh).host_operators()
    assert set(H) == set(D)
    for k in H:
        a, b = H[k], D[k]
        assert a.shape == b.shape, k
        assert np.array_equal(a.indptr, b.indptr) and np.array_equal(a.indices, b.indices), k
        np.testing.assert_allclose(b.data, a.data, rtol=0, atol=1e-13 * np.abs(a.data).max(), err_msg=k)


def test_device_assembly_is_deterministic():
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    from cupymag_gb300.workloads import tet_workload
    p, mesh = tet_workload(dict(n=6, jitter=0.2, axes=(0.3, 0.2, 0.15), ME=True, rot111=True, seed=2))
    a = SimulationOperators(p, assembly="device", mesh=mesh).host_operators()
    b = SimulationOperators(p, assembly="device", mesh=mesh).host_operators()
    for k in a:
        assert np.array_equal(a[k].data, b[k].data), k
