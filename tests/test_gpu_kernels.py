"""GPU kernels through the C-ABI against the CPU oracle / SciPy on the same inputs."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from . import _golden as G

pytestmark = pytest.mark.gpu


def _dev(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


@pytest.fixture(scope="module")
def golden_me():
    return G.load("hex_me_rot")


def test_spmv_matches_scipy(golden_me):
    from cupymag_gb300.utils.device_csr import DeviceCSR
    rng = np.random.default_rng(0)
    for name, A in G.matrices(golden_me).items():
        D = DeviceCSR.from_scipy(A)
        x = rng.normal(size=A.shape[1])
        y = (D @ _dev(x)).cpu().numpy()
        ref = A @ x
        np.testing.assert_allclose(y, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max(), err_msg=name)
        if A.shape[0] == A.shape[1]:
            X = rng.normal(size=(A.shape[1], 3))
            Y = (D @ _dev(X)).cpu().numpy()
            np.testing.assert_allclose(Y, A @ X, rtol=1e-13, atol=1e-13 * np.abs(A @ X).max(), err_msg=name)


def test_spmv_int64_rowptr_and_empty_rows():
    from cupymag_gb300.utils.device_csr import DeviceCSR
    rng = np.random.default_rng(1)
    A = sp.random(300, 200, density=0.05, random_state=2, format="csr")
    A[7, :] = 0.0
    A.eliminate_zeros()
    D = DeviceCSR.from_scipy(A)
    D64 = DeviceCSR(D.indptr.to(torch.int64), D.indices, D.data, D.shape)
    x = rng.normal(size=200)
    for M in (D, D64):
        np.testing.assert_allclose((M @ _dev(x)).cpu().numpy(), A @ x, rtol=1e-13, atol=1e-14)


def _spd(n=400, seed=0):
    rng = np.random.default_rng(seed)
    B = sp.random(n, n, density=0.02, random_state=seed)
    A = (B @ B.T + sp.eye(n) * 0.5).tocsr()
    return A, rng.normal(size=n)


def test_cg_matches_oracle_iterations():
    """Same recurrence and stopping rule as cupyx cg: iteration count within one, residual within tol."""
    from oracle.cg import cg as ocg
    from cupymag_gb300.solvers.linear_solvers import CGSolver, decode_info, new_info
    from cupymag_gb300.utils.device_csr import DeviceCSR
    for seed in range(3):
        A, b = _spd(seed=seed)
        rec = []
        xo, _ = ocg(A, b, tol=1e-10, maxiter=5000, record=rec)
        D = DeviceCSR.from_scipy(A)
        bd = _dev(b)
        x = torch.zeros_like(bd)
        info = new_info(1)
        CGSolver().launch(D, bd, x, info[0], tol=1e-10, maxiter=5000)
        inf = decode_info(info[0].cpu().numpy())
        assert inf["status"] == 0
        assert abs(inf["iters"][0] - rec[0]) <= 1, (inf["iters"][0], rec[0])
        xg = x.cpu().numpy()
        assert np.linalg.norm(b - A @ xg) <= 1e-10 * np.linalg.norm(b) * 1.0001
        # both are converged solutions: they agree to ~cond(A) * tol
        np.testing.assert_allclose(xg, xo, rtol=0, atol=1e-6 * np.abs(xo).max())


def test_cg_multi_rhs_equals_single(golden_me):
    from cupymag_gb300.solvers.linear_solvers import solve_cg
    A = G.matrix(golden_me, "A1")
    rng = np.random.default_rng(4)
    B = rng.normal(size=(A.shape[0], 3))
    B[:, 1] *= 1e-3
    X3 = solve_cg(A, B, tol=1e-10, maxiter=2000).cpu().numpy()
    for j in range(3):
        xj = solve_cg(A, B[:, j].copy(), tol=1e-10, maxiter=2000).cpu().numpy()
        assert np.array_equal(X3[:, j], xj), j


def test_cg_zero_rhs_and_warm_start(golden_me):
    from cupymag_gb300.solvers.linear_solvers import solve_cg
    A = G.matrix(golden_me, "A_demag")
    b = np.zeros(A.shape[0])
    x = solve_cg(A, b, x0=np.ones(A.shape[0]), use_init=True, tol=1e-10)
    assert torch.count_nonzero(x).item() == 0  # ||b|| == 0 returns b
    rng = np.random.default_rng(5)
    b = rng.normal(size=A.shape[0])
    b[0] = 0.0
    x1 = solve_cg(A, b, tol=1e-10, maxiter=5000).cpu().numpy()
    x2 = solve_cg(A, b, x0=x1, use_init=True, tol=1e-10, maxiter=5000).cpu().numpy()
    assert np.linalg.norm(A @ x2 - b) <= 1e-10 * np.linalg.norm(b) * 1.0001


def test_cg_not_converged_raises_reference_message(golden_me):
    from cupymag_gb300.solvers.linear_solvers import solve_cg
    A = G.matrix(golden_me, "A_el")
    b = np.random.default_rng(6).normal(size=A.shape[0])
    with pytest.raises(RuntimeError, match=r"Error! CG for elasticity did not converge. info=3, residual="):
        solve_cg(A, b, tol=1e-12, maxiter=3, system="elasticity")


def test_cg_mixed_precision_reaches_fp64_tolerance(golden_me):
    from cupymag_gb300.solvers.linear_solvers import solve_cg
    A = G.matrix(golden_me, "A_el")
    b = np.random.default_rng(7).normal(size=A.shape[0])
    b[[0, A.shape[0] // 3, 2 * A.shape[0] // 3]] = 0.0
    x = solve_cg(A, b, tol=1e-10, maxiter=20000, precision="IR").cpu().numpy()
    assert np.linalg.norm(b - A @ x) <= 1e-10 * np.linalg.norm(b) * 1.0001


def test_volume_average_matches_reference(golden_me):
    from cupymag_gb300.utils.volume_average import VolumeAverage
    g = golden_me
    Avg = VolumeAverage(g["node_coords"], g["elements"], g["global_id"])
    for key in ("f3", "f6", "f1"):
        got = Avg.compute_average_field_gpu(g["in_" + key]).cpu().numpy()
        np.testing.assert_allclose(got, g["out_avg_" + key], rtol=1e-12, atol=1e-15)
    got = Avg.compute_average_field_gpu(g["in_f3"], defect_flag=g["elements"][:, -1]).cpu().numpy()
    np.testing.assert_allclose(got, g["out_avg_f3_nodefect"], rtol=1e-12, atol=1e-15)


def test_eigenstrain_strain_hd_match_reference(golden_me):
    from cupymag_gb300.utils.compute_derivatives import ComputeDerivatives
    from cupymag_gb300.utils.device_csr import DeviceCSR
    from cupymag_gb300.utils.final_assembly import build_E0_from_m
    from cupymag_gb300.utils.rot_111_matrices import get_R_matrix
    g = golden_me
    p = G.params(g)
    n = int(g["n"])
    np.testing.assert_allclose(build_E0_from_m(p.lambda100, p.lambda111, g["in_m"]).cpu().numpy(), g["out_E0"],
                               rtol=1e-15, atol=0)
    F = [DeviceCSR.from_scipy(G.matrix(g, k)) for k in ("Fx", "Fy", "Fz")]
    D = ComputeDerivatives(*F)
    E = D.compute_E_from_u(n, g["in_u"]).cpu().numpy()
    np.testing.assert_allclose(E, g["out_E_from_u"], rtol=1e-12, atol=1e-12 * np.abs(g["out_E_from_u"]).max())
    ER = D.compute_E_from_u(n, g["in_u"], get_R_matrix()).cpu().numpy()
    np.testing.assert_allclose(ER, g["out_E_from_u_R"], rtol=1e-12, atol=1e-12 * np.abs(ER).max())
    Hd = torch.stack(D.compute_Hd_from_U(g["in_f1"]), dim=-1).cpu().numpy()
    np.testing.assert_allclose(Hd, g["out_Hd"], rtol=1e-12, atol=1e-12 * np.abs(Hd).max())
