"""Pin the CPU oracle against golden vectors produced by the reference's own code.

The fixtures in tests/golden/*.npz were written by tests/golden/make_golden.py,
which runs the unmodified reference sources (CuPy/Numba replaced by NumPy
stand-ins).  These tests check the oracle's mesh, periodic map, assembly,
volume average, eigenstrain, strain and LLG step against them.
"""
import numpy as np
import pytest

from oracle import assembly as OA
from oracle import mesh as OM
from oracle.llg import LLGState, M_matrix, R_matrix, build_E0, llg_step, strain_from_u
from oracle.volume_average import VolumeAverage

from . import _golden as G


def oracle_mesh(g, p):
    if p.grid_type == "Hex":
        coords, el = OM.hex_mesh(p.Nx, p.Ny, p.Nz, p.Ndx, p.Ndy, p.Ndz, p.defect_center)
        gid = OM.hex_periodic_map(p.Nx, p.Ny, p.Nz, coords)
    else:
        coords = g["tet_coords"]
        ind = OM.defect_indicator(p.defect_shape, p.defect_parameters, p.defect_rotation)
        el = OM.tet_elements(coords, g["tet_tets"], ind, p.defect_center)
        gid = OM.tet_periodic_map(coords)
    return coords, el, gid


def oracle_ops(g, p):
    coords, el, gid = oracle_mesh(g, p)
    n = int(gid.max()) + 1
    defect = OM.extract_defect_dofs(el, gid)
    C = OA.voigt_C(p.c11, p.c12, p.c44, p.rot111, M_matrix()) if p.ME else None
    ops = OA.build_operators(coords, el, gid, n, defect, p.alpha1, p.alpha2, ME=p.ME, C=C)
    return coords, el, gid, n, defect, ops


@pytest.fixture(scope="module", params=G.CASES)
def case(request):
    g = G.load(request.param)
    p = G.params(g)
    return request.param, g, p


def test_parameters(case):
    name, g, p = case
    for k, v in [("psi0", p.psi0), ("K1", p.K1), ("AA", p.AA), ("c11", p.c11), ("c12", p.c12), ("c44", p.c44),
                 ("s11", p.s11), ("s12", p.s12), ("s44", p.s44), ("elasC1", p.elasC1), ("elasC2", p.elasC2),
                 ("elasC3", p.elasC3), ("dt", p.dt), ("astar", p.astar), ("alpha", p.alpha),
                 ("Hext1", p.Hext[0]), ("Hext2", p.Hext[1]), ("Hext3", p.Hext[2]),
                 ("sigma11", p.sigma[0]), ("sigma22", p.sigma[1]), ("sigma12", p.sigma[3]),
                 ("sigma13", p.sigma[5]), ("stop_value", p.stop_value)]:
        assert g["param_" + k] == v, k
    np.testing.assert_array_equal(g["param_stop_direction"], p.stop_direction)


def test_mesh_and_dofs(case):
    name, g, p = case
    coords, el, gid = oracle_mesh(g, p)
    np.testing.assert_array_equal(coords, g["node_coords"])
    np.testing.assert_array_equal(el, g["elements"])
    np.testing.assert_array_equal(gid, g["global_id"])
    np.testing.assert_array_equal(OM.extract_defect_dofs(el, gid), g["DefDOF"])
    if p.grid_type == "Hex":
        i, j, k = np.meshgrid(np.arange(p.Nx + 1), np.arange(p.Ny + 1), np.arange(p.Nz + 1), indexing="ij")
        closed = (i % p.Nx) * p.Ny * p.Nz + (j % p.Ny) * p.Nz + (k % p.Nz)
        np.testing.assert_array_equal(closed.ravel(), gid)


def test_operators(case):
    name, g, p = case
    *_, ops = oracle_ops(g, p)
    gm = G.matrices(g)
    assert set(gm) == set(ops)
    for k, A in gm.items():
        B = ops[k]
        assert A.shape == B.shape, k
        np.testing.assert_array_equal(A.indptr, B.indptr, err_msg=k)
        np.testing.assert_array_equal(A.indices, B.indices, err_msg=k)
        scale = np.abs(A.data).max()
        np.testing.assert_allclose(B.data, A.data, rtol=0, atol=1e-13 * scale, err_msg=k)


def test_volume_average(case):
    name, g, p = case
    coords, el, gid = oracle_mesh(g, p)
    Avg = VolumeAverage(coords, el, gid)
    np.testing.assert_allclose(Avg.detJ, g["avg_detJ"], rtol=1e-14, atol=1e-14)
    np.testing.assert_allclose(Avg.N, g["avg_N"], rtol=0, atol=1e-16)
    for key in ["f3", "f6", "f1"]:
        np.testing.assert_allclose(Avg.average(g["in_" + key]), g["out_avg_" + key], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(Avg.average(g["in_f3"], defect_flag=el[:, -1]), g["out_avg_f3_nodefect"],
                               rtol=1e-12, atol=1e-15)
    # per-DOF weight form used by the device kernel
    n = int(gid.max()) + 1
    w, V = Avg.dof_weights(n)
    np.testing.assert_allclose(w @ g["in_f3"] / V, g["out_avg_f3"], rtol=1e-12, atol=1e-15)


def test_eigenstrain_strain_demag(case):
    name, g, p = case
    ops = G.matrices(g)
    n = int(g["n"])
    np.testing.assert_allclose(build_E0(p.lambda100, p.lambda111, g["in_m"]), g["out_E0"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(strain_from_u(ops, n, g["in_u"]), g["out_E_from_u"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(strain_from_u(ops, n, g["in_u"], R_matrix()), g["out_E_from_u_R"],
                               rtol=1e-13, atol=1e-13)
    Hd = np.stack([-(ops[k] @ g["in_f1"]) for k in ("Fx", "Fy", "Fz")], axis=-1)
    np.testing.assert_allclose(Hd, g["out_Hd"], rtol=1e-13, atol=1e-13)


def test_llg_steps(case):
    """The oracle's step on the reference's own operators reproduces main()'s loop."""
    name, g, p = case
    ops = G.matrices(g)
    coords, el, gid = oracle_mesh(g, p)
    Avg = VolumeAverage(coords, el, gid)
    defect = g["DefDOF"]
    m0 = g["m0"].copy()
    m0[defect] = 0.0
    S = LLGState(m0, Avg.average)
    K = g["step_m"].shape[0]
    for k in range(K):
        S.iters = []
        llg_step(S, ops, Avg.average, p, p.Hext, defect)
        its = [x for x in g["step_iters"][k] if x >= 0]
        assert S.iters == its, (k, S.iters, its)
        err = np.abs(S.m - g["step_m"][k]).max()
        assert err <= 1e-14, (k, err)
        np.testing.assert_allclose(S.avg_m, g["step_avg_m"][k], rtol=0, atol=1e-13)
        np.testing.assert_allclose(S.E, g["step_E"][k], rtol=0, atol=1e-12 * max(1.0, np.abs(g["step_E"][k]).max()))


def test_driver_sweep_matches_reference_main():
    """The reference's own convergence-driven sweep (main() run to its stop condition)."""
    from oracle.llg import run_driver
    g = G.load("hex_driver")
    p = G.params(g)
    ops = G.matrices(g)
    coords, el, gid = oracle_mesh(g, p)
    Avg = VolumeAverage(coords, el, gid)
    n = int(g["n"])
    v = np.asarray(p.initial_magnetization, dtype=np.float64)
    m0 = np.tile(v / np.linalg.norm(v), (n, 1))
    m0[g["DefDOF"]] = 0.0
    rows, m, steps = run_driver(p, ops, Avg.average, g["DefDOF"], m0)
    np.testing.assert_array_equal(rows[:, :3], g["hysteresis"][:, :3])
    np.testing.assert_allclose(rows[:, 3:], g["hysteresis"][:, 3:], rtol=0, atol=1e-14)
    np.testing.assert_allclose(m, g["final_m"], rtol=0, atol=1e-14)


def test_threaded_operators_give_the_oracle_step_bit_for_bit():
    """The CPU baseline's row-blocked threaded products and CG updates (oracle/threaded.py) leave the
    oracle's step and CG bit-identical to the single-threaded ones, and the blocks share the matrix's
    arrays."""
    import oracle.llg as OL
    from oracle.threaded import threaded_operators
    from oracle.volume_average import VolumeAverage as OVA
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    from cupymag_gb300.workloads import seeded_m0

    p = G.params(G.load("hex_me_rot"))
    S = SimulationOperators(p, device="cpu")
    ops = S.host_operators()
    tops, pool, threads = threaded_operators(ops, 4)
    try:
        blk = tops["A_el"].blocks[-1][2]
        assert np.shares_memory(blk.data, ops["A_el"].data)
        Avg = OVA(S.node_coords_np, S.elements_np, S.global_id_np)
        m0 = seeded_m0(S.n_dof, S.DefDOF, seed=5)
        out = []
        for o in (ops, tops):
            st = OL.LLGState(m0.copy(), Avg.average)
            for _ in range(2):
                OL.llg_step(st, o, Avg.average, p, p.Hext, S.DefDOF)
            out.append(st.m.copy())
        assert np.array_equal(out[0], out[1])
        # the CG with threaded element-wise updates, as the CPU baseline runs it
        from oracle.cg import cg
        from oracle.threaded import ThreadedAxpy
        b = np.random.default_rng(3).standard_normal(ops["A_el"].shape[0])
        b[[0, S.n_dof, 2 * S.n_dof]] = 0.0
        x1, i1 = cg(ops["A_el"], b, tol=1e-10, maxiter=400)
        x2, i2 = cg(tops["A_el"], b, tol=1e-10, maxiter=400, axpy=ThreadedAxpy(pool, threads))
        assert i1 == i2 and np.array_equal(x1, x2)
    finally:
        pool.shutdown()


def test_threaded_csr_with_64_bit_indices():
    """Row blocks of a CSR matrix with int64 indices (F_el at 192^3 needs them) keep the index type and
    the product's bits."""
    import scipy.sparse as sp
    from concurrent.futures import ThreadPoolExecutor
    from oracle.threaded import ThreadedCSR
    rng = np.random.default_rng(4)
    n, k = 5000, 7
    A = sp.csr_matrix((rng.standard_normal(n * k), rng.integers(0, n, n * k), np.arange(0, n * k + 1, k)),
                      shape=(n, n))
    A.indices = A.indices.astype(np.int64)
    A.indptr = A.indptr.astype(np.int64)
    with ThreadPoolExecutor(3) as pool:
        T = ThreadedCSR(A, pool, 3)
        assert all(b[2].indptr.dtype == np.int64 and b[2].indices.dtype == np.int64 for b in T.blocks)
        x = rng.standard_normal(n)
        X = rng.standard_normal((n, 3))
        assert np.array_equal(T @ x, A @ x) and np.array_equal(T @ X, A @ X)

