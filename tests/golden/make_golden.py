"""Generate golden vectors by running the reference's own Python sources.

The reference (CuPyMag) needs CuPy, a CUDA GPU, Numba, PyYAML, h5py, meshio and
pandas, none of which exist in the build container.  This script puts the
test-only stand-ins of ``_shims/`` in front of ``sys.path`` (cupy -> NumPy,
cupyx sparse -> SciPy, cupyx cg -> the oracle's restatement of CuPy's cg,
numba -> identity decorators, yaml -> json, h5py -> .npy) and then imports and
runs the reference's modules unmodified:

* ``cupymag.core.parameters`` -> nondimensional scalars;
* ``SimulationOperators`` -> every CSR operator, the volume-average tables,
  the periodic DOF map and the defect DOFs;
* ``build_E0_from_m``, ``ComputeDerivatives``, ``compute_average_field_gpu``
  on seeded inputs;
* ``Micromagnetics.main()`` for a few LLG steps (the step loop is cut after K
  steps by a stand-in ``stop_direction`` whose ``@`` records the loop state),
  and one case that runs main()'s own convergence-based field sweep to its
  stop condition and keeps ``hysteresis.txt`` and the final m.

Each case runs in a fresh subprocess because the reference loads its config
at import time.  Output: ``tests/golden/<case>.npz``.

Usage:  python tests/golden/make_golden.py --ref <reference checkout> [case ...]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent

MU0 = 1.25663706127e-6

BASE_PHYS = {
    "magnetic": {"ms": 1.2e6, "exchange_stiffness": 1.5e-11, "anisotropy_k1": 2.0e4},
    "elastic": {"c11": 196.0e9, "c12": 156.0e9, "c44": 123.0e9},
    "magnetostriction": {"lambda100": 2.0e-4, "lambda111": -2.0e-5},
    "demagnetization": {"n_x": 1 / 3, "n_y": 1 / 3, "n_z": 1 / 3},
    "external_field": {"hext1": 0.1 / MU0, "dhext1": 0.0, "hext2": 0.0, "dhext2": 0.0, "hext3": 0.0,
                       "dhext3": 0.0},
    "external_stress": {"sigma11": -50.0e6, "sigma22": 0.0, "sigma33": 0.0, "sigma12": 0.0, "sigma23": 0.0,
                        "sigma13": 0.0},
    "rotation_111": False,
    "magnetoelastic_coupling": False,
    "characteristic_length": 10.0e-9,
}

BASE_SIM = {
    "precision": "DP",
    "llg": {"timestep": 1.0e-12, "alpha_damping": 0.1, "llg_accuracy_factor": 5.0e-10},
    "solver": {"tolerance": 1.0e-10, "max_iterations": 20000, "initial_factor": 100.0},
    "restart": True,
    "restart_magnetization": None,
    "stop_condition": {"component": 0, "value": -0.95},
}


def _case_configs():
    def hexgrid(n, d, center=None):
        g = {"type": "Hex", "cubic_mesh": {"nx": n[0], "ny": n[1], "nz": n[2], "ndx": d[0], "ndy": d[1],
                                            "ndz": d[2]}}
        if center is not None:
            g["defect_center"] = center
        return g

    cases = {}
    # plain FP64, no ME (the 32^3 benchmark case in miniature)
    p = json.loads(json.dumps(BASE_PHYS))
    cases["hex_plain"] = dict(physics=p, grid=hexgrid((6, 6, 6), (2, 2, 2)), sim=BASE_SIM, steps=8, seed=11)
    # ME with the [111] rotation (the 128^3 benchmark case in miniature)
    p = json.loads(json.dumps(BASE_PHYS))
    p["magnetoelastic_coupling"] = True
    p["rotation_111"] = True
    cases["hex_me_rot"] = dict(physics=p, grid=hexgrid((6, 6, 6), (2, 2, 2)), sim=BASE_SIM, steps=5, seed=12)
    # ME without rotation, non-cubic box, off-centre defect, mixed stress
    p = json.loads(json.dumps(BASE_PHYS))
    p["magnetoelastic_coupling"] = True
    p["demagnetization"] = {"n_x": 0.0, "n_y": 0.0, "n_z": 1.0}
    p["external_field"].update({"hext2": 2000.0, "hext3": -500.0})
    p["external_stress"].update({"sigma22": 20.0e6, "sigma12": 5.0e6, "sigma13": -3.0e6})
    cases["hex_me_norot"] = dict(physics=p, grid=hexgrid((5, 6, 7), (2, 2, 3), center=[2.0, 3.5, 3.0]),
                                 sim=BASE_SIM, steps=4, seed=13)
    # tetrahedral mesh with a rotated ellipsoid defect, ME + rotation
    p = json.loads(json.dumps(BASE_PHYS))
    p["magnetoelastic_coupling"] = True
    p["rotation_111"] = True
    cases["tet_me_rot"] = dict(physics=p, grid={"type": "Tet"}, sim=BASE_SIM, steps=3, seed=14, tet=(3, 0.2))
    # the reference's own convergence-based field sweep, run to its stop condition
    p = json.loads(json.dumps(BASE_PHYS))
    p["external_field"].update({"hext1": 0.0, "dhext1": 15000.0})
    sim = json.loads(json.dumps(BASE_SIM))
    sim["llg"].update({"timestep": 3.0e-12, "alpha_damping": 0.5})
    sim["restart"] = False
    sim["initial_magnetization"] = [1.0, 0.02, 0.01]
    # no defect here: with non-magnetic cells the volume average can never reach the stop value
    cases["hex_driver"] = dict(physics=p, grid=hexgrid((4, 4, 4), (0, 0, 0)), sim=sim, steps=None, seed=15)
    return cases


def kuhn_tet_mesh(ne, jitter, seed):
    """A ne^3 cube of edge ne (h = 1) split into 6 Kuhn tets per cell, interior nodes jittered."""
    rng = np.random.default_rng(seed)
    g = np.arange(ne + 1, dtype=np.float64)
    I, J, K = np.meshgrid(g, g, g, indexing="ij")
    coords = np.stack([I.ravel(), J.ravel(), K.ravel()], axis=1)
    interior = np.all((coords > 0) & (coords < ne), axis=1)
    coords[interior] += rng.uniform(-jitter, jitter, size=(interior.sum(), 3))

    def nid(i, j, k):
        return (i * (ne + 1) + j) * (ne + 1) + k

    tets = []
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    for i in range(ne):
        for j in range(ne):
            for k in range(ne):
                for pm in perms:
                    cur = [i, j, k]
                    vs = [nid(*cur)]
                    for ax in pm:
                        cur = list(cur)
                        cur[ax] += 1
                        vs.append(nid(*cur))
                    p0, p1, p2, p3 = (coords[v] for v in vs)
                    if np.linalg.det(np.stack([p1 - p0, p2 - p0, p3 - p0])) < 0:
                        vs[1], vs[2] = vs[2], vs[1]
                    tets.append(vs)
    return coords, np.array(tets, dtype=np.int64)


def write_nas(path, coords, tets):
    with open(path, "w") as f:
        f.write("$ generated\n")
        for i, c in enumerate(coords):
            f.write(f"GRID,{i + 1},,{float(c[0])!r},{float(c[1])!r},{float(c[2])!r}\n")
        for e, t in enumerate(tets):
            f.write(f"CTETRA,{e + 1},1,{t[0] + 1},{t[1] + 1},{t[2] + 1},{t[3] + 1}\n")
        f.write("ENDDATA\n")


def seeded_rotation(seed):
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))[None, :]
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def run_case(name, ref, outdir):
    """Executed inside a fresh subprocess."""
    cfg = _case_configs()[name]
    tmp = Path(tempfile.mkdtemp(prefix=f"golden_{name}_"))
    grid = dict(cfg["grid"])
    extra = {}
    if grid["type"] == "Tet":
        ne, jit = cfg["tet"]
        coords, tets = kuhn_tet_mesh(ne, jit, cfg["seed"])
        nas = tmp / "mesh.nas"
        write_nas(nas, coords, tets)
        Rd = seeded_rotation(cfg["seed"] + 100)
        grid["tet_mesh"] = {"mesh_file": str(nas), "defect_shape": "RotatedEllipsoid",
                            "defect_parameters": [1.0, 0.7, 0.5], "rotation_matrix": Rd.tolist()}
        extra["tet_coords"] = coords
        extra["tet_tets"] = tets
        extra["tet_defect_rotation"] = Rd
    sim = json.loads(json.dumps(cfg["sim"]))
    if sim.get("restart"):
        sim["restart_magnetization"] = str(tmp / "m0.h5")
    config = {"physics": cfg["physics"], "grid": grid, "simulation": sim,
              "output": {"directory": str(tmp), "write_magnetization": True, "save_frequency": 100000,
                         "vtu_blend_alpha": 0.05}}
    cpath = tmp / "config.yaml"
    cpath.write_text(json.dumps(config, indent=1))
    sys.argv = [sys.argv[0]]
    os.environ["CUPYMAG_CONFIG_PATH"] = str(cpath)
    sys.path[:0] = [str(HERE / "_shims"), str(ref), str(REPO)]

    import cupymag.core.parameters as P
    from cupymag.core.assemble_simulation_operators import SimulationOperators
    from cupymag.mesh.setup_FEM_mesh import FEMMesh
    from cupymag.utils.final_assembly import build_E0_from_m
    from cupymag.utils.volume_average import VolumeAverage
    import cupyx.scipy.sparse.linalg as spla

    out = {"config_json": np.array(json.dumps(config))}
    for k in ["psi0", "K1", "AA", "c11", "c12", "c44", "s11", "s12", "s44", "elasC1", "elasC2", "elasC3",
              "dt", "astar", "alpha", "Hext1", "Hext2", "Hext3", "dHext1", "dHext2", "dHext3", "sigma11",
              "sigma22", "sigma33", "sigma12", "sigma23", "sigma13", "stop_value"]:
        out["param_" + k] = np.float64(getattr(P, k))
    out["param_stop_direction"] = np.asarray(P.stop_direction, dtype=np.float64)

    S = SimulationOperators()
    n = S.n_dof
    out["n"] = np.int64(n)
    out["node_coords"] = np.asarray(S.node_coords_np)
    out["elements"] = np.asarray(S.elements_np)
    out["global_id"] = np.asarray(S.global_id_np)
    out["DefDOF"] = np.asarray(S.DefDOF)
    A_demag, Fx, Fy, Fz, Deriv = S.csr_demag_and_deriv()
    A1, A2, F1 = S.csr_GS()
    A_el, F_el = S.csr_elasticity()
    mats = {"A_demag": A_demag, "Fx": Fx, "Fy": Fy, "Fz": Fz, "A1": A1, "A2": A2, "F1": F1}
    if A_el is not None:
        mats.update({"A_el": A_el, "F_el": F_el})
    for k, A in mats.items():
        out[f"mat_{k}_data"] = np.asarray(A.data)
        out[f"mat_{k}_indices"] = np.asarray(A.indices)
        out[f"mat_{k}_indptr"] = np.asarray(A.indptr)
        out[f"mat_{k}_shape"] = np.asarray(A.shape)
    Avg = S.volume_average()
    out["avg_detJ"] = np.asarray(Avg.detJ)
    out["avg_N"] = np.asarray(Avg.N_gauss_gpu)
    out["avg_corner_dofs"] = np.asarray(Avg.corner_dofs)

    rng = np.random.default_rng(cfg["seed"])
    f3 = rng.normal(size=(n, 3))
    f6 = rng.normal(size=(n, 6))
    f1 = rng.normal(size=n)
    out["in_f3"], out["in_f6"], out["in_f1"] = f3, f6, f1
    out["out_avg_f3"] = np.asarray(Avg.compute_average_field_gpu(f3))
    out["out_avg_f6"] = np.asarray(Avg.compute_average_field_gpu(f6))
    out["out_avg_f1"] = np.asarray(Avg.compute_average_field_gpu(f1))
    dfl = np.asarray(S.elements_np)[:, -1]
    out["out_avg_f3_nodefect"] = np.asarray(Avg.compute_average_field_gpu(f3, defect_flag=dfl))
    mrand = rng.normal(size=(n, 3))
    mrand /= np.linalg.norm(mrand, axis=1, keepdims=True)
    out["in_m"] = mrand
    out["out_E0"] = np.asarray(build_E0_from_m(P.lambda100, P.lambda111, mrand))
    u = rng.normal(size=3 * n)
    out["in_u"] = u
    out["out_E_from_u"] = np.asarray(Deriv.compute_E_from_u(n, u))
    from cupymag.utils.rot_111_matrices import get_R_matrix
    R = get_R_matrix(backend="numpy")
    out["out_E_from_u_R"] = np.asarray(Deriv.compute_E_from_u(n, u, R))
    Hd = Deriv.compute_Hd_from_U(f1)
    out["out_Hd"] = np.stack([np.asarray(h) for h in Hd], axis=-1)

    # ---- LLG steps through the reference's own main() ----
    FEMMesh._mesh_computed = False
    FEMMesh.DefDOF = None
    VolumeAverage.write_to_paraview = lambda *a, **k: None
    import cupymag.core.Micromagnetics as MM

    if cfg["steps"] is not None:
        m0 = np.array([1.0, 0.0, 0.0]) + rng.normal(0.0, 1e-3, size=(n, 3))
        m0 /= np.linalg.norm(m0, axis=1, keepdims=True)
        np.save(str(tmp / "m0.h5") + ".npy", m0)
        out["m0"] = m0
        K = cfg["steps"]
        rec = {"m": [], "avg_m": [], "E": [], "iters": []}

        class Probe:
            __array_ufunc__ = None

            def __init__(self):
                self.calls = 0

            def __rmatmul__(self, avg_m):
                frame = sys._getframe(1)
                loc = frame.f_locals
                if self.calls > 0:
                    rec["m"].append(np.array(loc["m"], dtype=np.float64))
                    rec["avg_m"].append(np.array(avg_m, dtype=np.float64))
                    rec["E"].append(np.array(frame.f_globals["E"], dtype=np.float64))
                    rec["iters"].append(list(spla.CG_LOG))
                spla.CG_LOG.clear()
                self.calls += 1
                return 1.0 if self.calls <= K else -1.0

        MM.stop_direction = Probe()
        MM.main()
        out["step_m"] = np.stack(rec["m"])
        out["step_avg_m"] = np.stack(rec["avg_m"])
        out["step_E"] = np.stack(rec["E"])
        its = rec["iters"]
        width = max(len(x) for x in its)
        out["step_iters"] = np.array([x + [-1] * (width - len(x)) for x in its])
    else:
        MM.main()
        out["hysteresis"] = np.loadtxt(tmp / "hysteresis.txt", skiprows=1)
        out["final_m"] = np.load(str(tmp / "last_m.h5") + ".npy")
    out.update(extra)
    np.savez_compressed(Path(outdir) / f"{name}.npz", **out)
    print(f"wrote {name}.npz")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the reference checkout (its cupymag/ package)")
    ap.add_argument("--case", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--outdir", default=str(HERE))
    ap.add_argument("cases", nargs="*")
    a = ap.parse_args()
    if a.case:
        run_case(a.case, a.ref, a.outdir)
        return
    names = a.cases or list(_case_configs())
    for nm in names:
        r = subprocess.run([sys.executable, __file__, "--ref", a.ref, "--case", nm, "--outdir", a.outdir],
                           capture_output=True, text=True)
        if r.returncode != 0:
            print(r.stdout[-3000:])
            print(r.stderr[-5000:])
            raise SystemExit(f"case {nm} failed")
        print(r.stdout.strip().splitlines()[-1])


if __name__ == "__main__":
    main()
