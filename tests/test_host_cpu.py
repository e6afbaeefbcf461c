"""CPU tests of the host side: config loader, parameters, mesh, assembly, C-ABI exports."""
import os
import re

import numpy as np
import pytest

from . import _golden as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# ------------------------------------------------------------------ YAML subset / parameters
def test_yaml_subset_pyyaml_resolution():
    from cupymag_gb300.core.config_loader import safe_load
    d = safe_load(
        "a: 1.25e+6  # float\nb: 1e6\nc: 1.0e6\nd: 10.0e-9\ne: [[1.0, 0.0], [0, 1]]\nf: yes\ng: 'q # x'\n"
        "h:\n  - 1\n  - k: 2\n    l: 3\ni: ~\nj: \"s\"\nk: .5\nl: -0.95\nm: 0x1f\n")
    assert d["a"] == 1.25e6 and d["b"] == "1e6" and d["c"] == "1.0e6" and d["d"] == 10.0e-9
    assert d["e"] == [[1.0, 0.0], [0, 1]] and d["f"] is True and d["g"] == "q # x"
    assert d["h"] == [1, {"k": 2, "l": 3}] and d["i"] is None and d["j"] == "s" and d["k"] == 0.5
    assert d["l"] == -0.95 and d["m"] == 31


def test_example_config_parses(tmp_path):
    from cupymag_gb300.core.parameters import load_parameters
    cfg = """
physics:
  magnetic:
    ms: 1.25e+6
    exchange_stiffness: 1.0e-11
    anisotropy_k1: 958.0
  elastic: {c11: 240.0e+9, c12: 89.0e+9, c44: 76.0e+9}
  magnetostriction:
    lambda100: 10.0e-6
    lambda111: 30.9e-6
  demagnetization: {n_x: 0.0, n_y: 0.0, n_z: 1.0}
  external_field: {hext1: 200.0, dhext1: 20.0, hext2: 0.01}
  external_stress: {sigma11: 0.0}
  rotation_111: false
  magnetoelastic_coupling: true
  characteristic_length: 10.0e-9
grid:
  type: "Hex"
  cubic_mesh: {nx: 8, ny: 8, nz: 4, ndx: 2, ndy: 2, ndz: 2}
simulation:
  precision: "DP"
  llg: {timestep: 3.0e-12, alpha_damping: 0.15, llg_accuracy_factor: 5.0e-10}
  solver: {tolerance: 1.0e-7, max_iterations: 5000, initial_factor: 100.0}
  restart: false
  initial_magnetization: [1.0, 0.0, 0.0]
  stop_condition:
    direction: [0.8, 0.6, 0.0]
    value: -0.95
output:
  directory: "out"
"""
    p = tmp_path / "c.yaml"
    p.write_text(cfg)
    P = load_parameters(p)
    assert P.Nx == 8 and P.Nz == 4 and P.ME and not P.rot111
    np.testing.assert_allclose(P.stop_direction, (0.8, 0.6, 0.0))
    assert P.output_dir == str((tmp_path / "out").resolve())
    assert P.dt == pytest.approx(3e-12 * 1.25663706127e-6 * 1.76e11 * 1.25e6 / (1 + 0.15 ** 2), rel=1e-15)


def test_parameter_validation():
    from cupymag_gb300.core.parameters import SimParams
    with pytest.raises(ValueError, match="Saturation magnetization must be positive"):
        SimParams(ms=0.0).finalize()
    with pytest.raises(ValueError, match="Timestep must be positive"):
        SimParams(timestep=0.0).finalize()


@pytest.mark.parametrize("case", G.CASES)
def test_parameters_match_reference(case):
    g = G.load(case)
    p = G.params(g)
    for k in ["dt", "alpha", "K1", "elasC1", "elasC2", "elasC3", "s11", "s12", "s44"]:
        assert getattr(p, k) == g["param_" + k], k


# ------------------------------------------------------------------ mesh / assembly
@pytest.mark.parametrize("case", G.CASES)
def test_mesh_and_coo_assembly_match_reference(case):
    from cupymag_gb300.mesh.grids import HexGrid, TetraGrid, extract_defect_dofs
    from cupymag_gb300.physics.assembly import assemble_coo, stiffness_voigt
    from cupymag_gb300.utils.defect_shapes import get_defect_shape_function
    from cupymag_gb300.utils.rot_111_matrices import get_M_matrix
    g = G.load(case)
    p = G.params(g)
    if p.grid_type == "Hex":
        grid = HexGrid(p.Nx, p.Ny, p.Nz, p.Ndx, p.Ndy, p.Ndz, p.defect_center)
    else:
        fn = get_defect_shape_function(p.defect_shape, (p.defect_parameters, p.defect_rotation))
        grid = TetraGrid(coords=g["tet_coords"], tets=g["tet_tets"], defect_shape=fn)
    coords, el = grid.std_fem_mesh()
    gid = grid.build_periodic_node_map(coords)
    np.testing.assert_array_equal(coords, g["node_coords"])
    np.testing.assert_array_equal(el, g["elements"])
    np.testing.assert_array_equal(gid, g["global_id"])
    D = extract_defect_dofs(el, gid)
    np.testing.assert_array_equal(D, g["DefDOF"])
    if p.grid_type == "Hex":
        np.testing.assert_array_equal(grid.defect_dofs(), D)
    C = stiffness_voigt(p.c11, p.c12, p.c44, get_M_matrix() if p.rot111 else None)
    ops = assemble_coo(coords, el, gid, int(gid.max()) + 1, D, p.alpha1, p.alpha2, p.ME, C)
    for k, A in G.matrices(g).items():
        B = ops[k]
        np.testing.assert_array_equal(A.indptr, B.indptr, err_msg=k)
        np.testing.assert_array_equal(A.indices, B.indices, err_msg=k)
        np.testing.assert_allclose(B.data, A.data, rtol=0, atol=1e-14 * np.abs(A.data).max(), err_msg=k)


@pytest.mark.parametrize("case", ["hex_plain", "hex_me_rot", "hex_me_norot"])
def test_structured_hex_assembly_matches_reference(case):
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    g = G.load(case)
    p = G.params(g)
    ops = SimulationOperators(p, device="cpu", assembly="structured").host_operators()
    for k, A in G.matrices(g).items():
        B = ops[k]
        np.testing.assert_array_equal(A.indptr, B.indptr, err_msg=k)
        np.testing.assert_array_equal(A.indices, B.indices, err_msg=k)
        np.testing.assert_allclose(B.data, A.data, rtol=0, atol=2e-15 * np.abs(A.data).max(), err_msg=k)


def test_structured_equals_coo_on_larger_grid():
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    p = G.params(G.load("hex_me_rot")).with_(Nx=7, Ny=5, Nz=9, Ndx=3, Ndy=2, Ndz=4)
    a = SimulationOperators(p, device="cpu", assembly="structured").host_operators()
    b = SimulationOperators(p, device="cpu", assembly="coo").host_operators()
    for k in a:
        np.testing.assert_array_equal(a[k].indptr, b[k].indptr, err_msg=k)
        np.testing.assert_array_equal(a[k].indices, b[k].indices, err_msg=k)
        np.testing.assert_allclose(a[k].data, b[k].data, rtol=0, atol=2e-15 * np.abs(b[k].data).max(), err_msg=k)


def test_periodic_map_matches_reference_loop():
    from oracle.mesh import tet_periodic_map
    from cupymag_gb300.mesh.grids import TetraGrid, kuhn_tet_cube
    coords, tets = kuhn_tet_cube(4, jitter=0.2, seed=3)
    np.testing.assert_array_equal(TetraGrid(coords=coords, tets=tets).build_periodic_node_map(),
                                  tet_periodic_map(coords))


def test_nas_roundtrip(tmp_path):
    from cupymag_gb300.mesh.grids import kuhn_tet_cube, read_nas, write_nas
    coords, tets = kuhn_tet_cube(3, jitter=0.2, seed=1)
    f = tmp_path / "m.nas"
    write_nas(f, coords, tets)
    ids, c2, eids, t2 = read_nas(f)
    np.testing.assert_array_equal(c2, coords)
    np.testing.assert_array_equal(t2, tets)
    p = coords[tets]
    assert (np.linalg.det(p[:, 1:] - p[:, :1]) > 0).all()


def test_volume_average_weights_match_reference():
    from cupymag_gb300.utils.volume_average import dof_weights
    for case in G.CASES:
        g = G.load(case)
        w, V = dof_weights(g["node_coords"], g["elements"], g["global_id"], int(g["n"]))
        np.testing.assert_allclose(w @ g["in_f3"] / V, g["out_avg_f3"], rtol=1e-12, atol=1e-15)
        w2, V2 = dof_weights(g["node_coords"], g["elements"], g["global_id"], int(g["n"]),
                             defect_flag=g["elements"][:, -1])
        np.testing.assert_allclose(w2 @ g["in_f3"] / V2, g["out_avg_f3_nodefect"], rtol=1e-12, atol=1e-15)


# ------------------------------------------------------------------ C-ABI
def _header_functions():
    txt = open(os.path.join(ROOT, "include", "cupymag_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cpm_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_header_symbol():
    from cupymag_gb300 import _native as N
    from cupymag_gb300.build import build
    build()
    lib = N.load()
    names = _header_functions()
    assert names, "no functions parsed from the header"
    for nm in names:
        assert hasattr(lib, nm), nm
    assert set(names) <= set(N.EXPORTED) | {"cpm_device_sm_count"}
    assert lib.cpm_version().startswith(b"cupymag_gb300")
    assert lib.cpm_cg_workspace_bytes(1000, 3, 1) > lib.cpm_cg_workspace_bytes(10, 1, 1)


def test_ctypes_structs_match_the_header_layouts(tmp_path):
    """Every ctypes mirror in _native has the size and field offsets of its C struct in
    include/cupymag_gb300.h, as gcc lays them out (a drifted field would pass wrong values silently)."""
    import ctypes
    import shutil
    import subprocess
    from cupymag_gb300 import _native as N
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    mirrors = {"cpm_csr": N.CSR, "cpm_cg_info": N.CGInfo, "cpm_cg_opts": N.CGOpts, "cpm_stencil": N.Stencil,
               "cpm_batch_system": N.BatchSystem, "cpm_batch_plan": N.BatchPlan, "cpm_field_params": N.FieldParams,
               "cpm_fft_precond": N.FftPrecondC, "cpm_deriv_stencil": N.DerivStencilC,
               "cpm_fel_stencil": N.FelStencilC}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "cupymag_gb300.h"', 'int main(void) {']
    for cname, py in mirrors.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_batch_work_bytes_follow_the_grid():
    """cpm_batch_work_bytes sizes a system's work vectors from its grid (host arithmetic, no GPU)."""
    from cupymag_gb300 import _native as N
    from cupymag_gb300.build import build
    from cupymag_gb300.serving.blockdiag import work_bytes
    build()
    N.load()
    al = lambda b: (b + 255) // 256 * 256  # noqa: E731
    assert work_bytes((10, 11, 12), 3, 1, "IR") == 5 * al(10 * 11 * 12 * 3 * 4)   # r, p, q (w), d, s in FP32
    assert work_bytes((10, 11, 12), 1, 3, "DP") == 3 * al(10 * 11 * 12 * 3 * 8)   # r, p, q in FP64
    assert work_bytes((9, 9, 9), 1, 1, "IR") == 5 * al(729 * 4)
    for dims, ncomp, nrhs in (((0, 4, 4), 1, 1), ((4, 4, 4), 2, 1), ((4, 4, 4), 1, 2)):
        with pytest.raises(ValueError):
            work_bytes(dims, ncomp, nrhs, "IR")


def test_fp32_product_rejects_what_its_form_cannot_take():
    """cpm_stencil_apply32 checks its arguments on the host before any launch (no GPU needed)."""
    from cupymag_gb300 import _native as N
    from cupymag_gb300.build import build
    build()
    lib = N.load()
    s = N.Stencil()
    s.nx, s.ny, s.nz, s.ncomp = 5, 5, 7, 1
    s.flags = None
    fake = 1 << 20  # a device address that the rejected calls never touch
    assert lib.cpm_stencil_apply32(s, fake, fake, 1, 1, None) == N.CPM_BAD_ARG   # nz = 7: no aligned quads
    assert "form 1 needs nz % 4 == 0" in N.last_error()
    for nvec, form in ((1, 3), (1, -1), (2, 0)):
        assert lib.cpm_stencil_apply32(s, fake, fake, nvec, form, None) == N.CPM_BAD_ARG, (nvec, form)
    s.ncomp = 3
    assert lib.cpm_stencil_apply32(s, fake, fake, 3, 0, None) == N.CPM_BAD_ARG   # elastic takes one vector
    s.nz = 2
    assert lib.cpm_stencil_apply32(s, fake, fake, 1, 0, None) == N.CPM_BAD_ARG   # fewer than 3 cells
    assert lib.cpm_stencil_apply32(None, fake, fake, 1, 0, None) == N.CPM_BAD_ARG


def test_double_float_error_bound_uses_the_symbol_minimum():
    """cpm_stencil_df_error_bound (host only): 2 g sum|c| / sigma_min with g = 128 * 2^-48, sigma_min
    taken at the 8 corners of the torus for stencils even along every axis.  Checked against the symbol's
    minimum on a fine grid of wave vectors for the Gauss-Seidel operators A1 and A2 (Q = sum|c| / sigma_min
    near 10.5 and 23.3) and the mass matrix (Q = 27); none for the demag operator (sigma(0) = 0) or an
    elastic stencil; a stencil that is not even along an axis gets a larger bound, never a smaller one."""
    import itertools
    from cupymag_gb300 import _native as N
    from cupymag_gb300.build import build
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    from cupymag_gb300.physics import structured_hex as SH
    build()
    lib = N.load()
    g = 128.0 * 2.0 ** -48
    p = G.params(G.load("hex_me_rot")).with_(Nx=8, Ny=8, Nz=8, Ndx=2, Ndy=2, Ndz=2)
    S = SimulationOperators(p, device="cpu")
    e = S._cell()
    th = np.linspace(0.0, 2 * np.pi, 41)

    def symbol_min(c):
        c = c.reshape(3, 3, 3)
        cx, cy, cz = (np.cos(np.multiply.outer(th, [-1.0, 0.0, 1.0])) for _ in range(3))
        sig = np.einsum("abc,ia,jb,kc->ijk", c, cx, cy, cz)  # even stencils: a product of cosines
        return sig.min()

    def bound(c, ncomp=1):
        s = N.Stencil()
        s.nx = s.ny = s.nz = 8
        s.ncomp = ncomp
        s.coef[:c.size] = tuple(float(v) for v in c)
        s.flags = None
        return lib.cpm_stencil_df_error_bound(s)

    for name, K, q in (("A1", e["K"] * S.alpha1 + e["M"], 10.5), ("A2", e["K"] * S.alpha2 + e["M"], 23.3),
                       ("M", e["M"], 27.0)):
        c = SH.stencil_from_element(K).reshape(-1)
        corners = min(np.einsum("abc,a,b,c->", c.reshape(3, 3, 3), *[np.array([u, 1.0, u]) for u in us])
                      for us in itertools.product((1.0, -1.0), repeat=3))
        assert abs(corners - symbol_min(c)) <= 1e-12 * np.abs(c).sum(), name
        got = bound(c)
        assert got == pytest.approx(2 * g * np.abs(c).sum() / corners, rel=1e-12), name
        assert abs(np.abs(c).sum() / corners - q) < 0.1, name
        assert got <= 0.25 * 1e-10, name
        # an odd part along x: the bound grows by the odd part's magnitude in the denominator
        odd = c.reshape(3, 3, 3).copy()
        odd[0] += 1e-3 * np.abs(c).max()
        assert bound(odd.reshape(-1)) > got, name
    assert bound(SH.stencil_from_element(e["K"]).reshape(-1)) == -1.0
    assert bound(SH.stencil_from_element(e["Kel"], 3, 3).reshape(-1), ncomp=3) == -1.0
    assert lib.cpm_stencil_df_error_bound(None) == -1.0


def _df_fma(w, x, acc):
    """float32 emulation of the device's double-float acc + w x (csrc/stencil_ops.cuh, df::fma); each
    operand is a (hi, lo) pair of float32 arrays.  A float32 product is exact in float64, so the FMAs are
    the float64 expression rounded once to float32."""
    f32, f64 = np.float32, np.float64
    (wh, wl), (xh, xl), (ah, al) = w, x, acc
    p = wh * xh
    e = (wh.astype(f64) * xh - p).astype(f32)
    e = (wh.astype(f64) * xl + e).astype(f32)
    e = (wl.astype(f64) * xh + e).astype(f32)
    s = ah + p
    bv = s - ah
    err = (ah - (s - bv)) + (p - bv)
    low = al + (err + e)
    h = s + low
    return h, low - (h - s)


def test_double_float_row_sum_stays_within_its_proven_bound():
    """27-term rows of the Gauss-Seidel stencil in the double-float arithmetic of the residual passes
    (emulated in float32): every row's sum is within 96 * 2^-48 of the sum of its terms' magnitudes of the
    exact sum (94 for the arithmetic, 2 for splitting c and x into float pairs), on smooth, constant
    (maximal cancellation) and random operands, far inside the g = 128 * 2^-48 that the bound uses."""
    from fractions import Fraction
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    from cupymag_gb300.physics import structured_hex as SH
    p = G.params(G.load("hex_me_rot")).with_(Nx=8, Ny=8, Nz=8, Ndx=2, Ndy=2, Ndz=2)
    S = SimulationOperators(p, device="cpu")
    e = S._cell()
    c = SH.stencil_from_element(e["K"] * S.alpha2 + e["M"]).reshape(-1)
    rng = np.random.default_rng(5)
    rows = 400
    t = np.linspace(0, 1, 27)
    xs = np.concatenate([1.0 + 1e-3 * np.sin(7 * t)[None, :] * rng.normal(size=(rows // 4, 1)),
                         np.full((rows // 4, 27), 0.731),
                         rng.normal(size=(rows // 2, 27)) * 10.0 ** rng.integers(-3, 3, size=(rows // 2, 1))])

    def split(v):
        hi = v.astype(np.float32)
        return hi, (v - hi.astype(np.float64)).astype(np.float32)

    ch, cl = split(np.broadcast_to(c, xs.shape))
    xh, xl = split(xs)
    acc = (np.zeros(rows, np.float32), np.zeros(rows, np.float32))
    for d in range(27):
        acc = _df_fma((ch[:, d], cl[:, d]), (xh[:, d], xl[:, d]), acc)
    got = acc[0].astype(np.float64) + acc[1].astype(np.float64)
    worst = 0.0
    for r in range(rows):
        exact = sum(Fraction(float(c[d])) * Fraction(float(xs[r, d])) for d in range(27))
        mag = float(sum(abs(Fraction(float(c[d])) * Fraction(float(xs[r, d]))) for d in range(27)))
        err = abs(float(Fraction(float(got[r])) - exact))
        worst = max(worst, err / (mag * 2.0 ** -48))
    assert worst <= 96.0, worst
    print("largest row error in units of 2^-48 sum|terms|:", worst)


# ------------------------------------------------------------------ serving (host side)
def test_serving_workload_shape():
    from cupymag_gb300.serving.workload import serving_requests
    reqs = serving_requests()
    assert len(reqs) == 256
    edges = np.array([r.edge for r in reqs])
    assert edges.min() >= 16 and edges.max() <= 96
    assert all(0 <= r.defect <= r.edge // 4 for r in reqs)
    assert sum(r.ME for r in reqs) == 128
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) >= 0) and arr[0] == 0.0
    assert 15.0 < (len(arr) - 1) / arr[-1] < 25.0
    assert all(0.05 <= r.B0 <= 0.2 and r.steps == 100 for r in reqs)
    # log-uniform edges: about half below the geometric mean of 16 and 96
    assert 0.35 < np.mean(edges < np.sqrt(16 * 96)) < 0.65
    assert serving_requests()[17] == reqs[17]


def test_serving_field_schedule():
    from cupymag_gb300.core.constants import MU0
    from cupymag_gb300.serving.workload import Request
    r = Request(0, 16, 2, False, 0.1, 5, 1)
    p = r.params()
    f = r.fields(p)
    assert f.shape == (5, 3)
    np.testing.assert_allclose(f[0, 0] * p.ms * MU0, 0.1)
    np.testing.assert_allclose(f[-1, 0] * p.ms * MU0, -0.1)
    assert np.all(f[:, 1:] == 0)


def test_memory_estimate_grows_with_size_and_coupling():
    from cupymag_gb300.serving.engine import estimate_bytes
    from cupymag_gb300.workloads import hex_params
    a = estimate_bytes(hex_params(32, 4, False, False))
    b = estimate_bytes(hex_params(32, 4, True, True))
    c = estimate_bytes(hex_params(64, 4, True, True))
    assert a < b < c
    # matrix-free operators: about 500 bytes per DOF at 96^3 with coupling
    assert 0.3e9 < estimate_bytes(hex_params(96, 12, True, True)) < 0.8e9


def test_flags_mark_neighbours_of_excluded_and_of_unpinned_columns():
    """Bit 8 on the 27-point neighbourhood of every excluded column, bit 16 only around excluded
    columns whose rows are not identity rows (pinned DOFs, flags 1|4, need no column tests in the
    FP32 refinement solver)."""
    from cupymag_gb300.utils.stencil_operator import (COL_EXCLUDED, NEAR_EXCLUDED, NEAR_UNPINNED, ROW_IDENTITY,
                                                      StencilOperator)
    nx = ny = nz = 6
    n = nx * ny * nz
    f = np.zeros(n, dtype=np.uint8)
    node = lambda i, j, k: (i * ny + j) * nz + k  # noqa: E731
    f[node(0, 0, 0)] = ROW_IDENTITY | COL_EXCLUDED      # pinned (wraps around the periodic grid)
    f[node(3, 3, 3)] = COL_EXCLUDED                     # excluded column, regular row
    S = StencilOperator(nx, ny, nz, np.ones(27), f, device="cpu")
    g = S.flags.numpy()
    near_pin = {node(i % nx, j % ny, k % nz) for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)}
    near_free = {node(3 + i, 3 + j, 3 + k) for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)}
    for d in range(n):
        assert bool(g[d] & NEAR_EXCLUDED) == (d in near_pin or d in near_free), d
        assert bool(g[d] & NEAR_UNPINNED) == (d in near_free), d
    assert S.anchor == -1
    pin_only = np.zeros(n, dtype=np.uint8)
    pin_only[node(2, 1, 4)] = ROW_IDENTITY | COL_EXCLUDED
    assert StencilOperator(nx, ny, nz, np.ones(27), pin_only, device="cpu").anchor == node(2, 1, 4)
