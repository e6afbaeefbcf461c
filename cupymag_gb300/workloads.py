"""Synthetic benchmark workloads (the reference publishes no datasets).

Every workload is a seeded synthetic LLG run; unspecified choices (ld = 10 nm,
rot111 off for the 32^3 case and on for the magnetoelastic cases, tol 1e-10,
maxiter 20000, llg_accuracy_factor 5e-10, initial_factor 100) are fixed here
and recorded in every bench line.

* hex32_plain:     32^3 hex, 4^3 defect, no ME, 500-step sweep +0.1 T -> -0.1 T.
* hex128_me:       128^3 hex, 16^3 defect, ME + [111] rotation, sigma_xx = -50 MPa,
                   c11/c12/c44 = 196/156/123 GPa, lambda100 = 2e-4, lambda111 = -2e-5.
* hex256_plain / hex192_me: the two halves of the precision-form case.
* tet96_me:        96^3 cube of Kuhn tets, interior nodes jittered +-0.2 h,
                   rotated ellipsoidal defect (semi-axes 0.15, 0.10, 0.08 of the edge).
Field schedule: H1_s = (B0 - 2 B0 s/(S-1)) / mu0, normalised by Ms.
Initial state: normalise((1,0,0) + N(0, 1e-3)) from numpy.random.default_rng(seed).
"""
from __future__ import annotations

import numpy as np

from .core.constants import MU0
from .core.parameters import SimParams

MAGNETIC = dict(ms=1.2e6, AA_raw=1.5e-11, K1_raw=2.0e4, N_x=1 / 3, N_y=1 / 3, N_z=1 / 3, alpha_damp=0.1,
                timestep=1e-12, ld=10.0e-9, tol=1e-10, maxiter=20000, LLG_accuracy_factor=5e-10,
                use_init_factor=100.0, precision="DP")
ELASTIC = dict(c11_raw=196.0e9, c12_raw=156.0e9, c44_raw=123.0e9, lambda100=2.0e-4, lambda111=-2.0e-5,
               sigma_raw=(-50.0e6, 0.0, 0.0, 0.0, 0.0, 0.0))


def hex_params(n, defect, ME, rot111, **kw) -> SimParams:
    p = SimParams(**MAGNETIC)
    if ME:
        for k, v in ELASTIC.items():
            setattr(p, k, v)
    p.grid_type = "Hex"
    p.Nx = p.Ny = p.Nz = n
    p.Ndx = p.Ndy = p.Ndz = defect
    p.ME = ME
    p.rot111 = rot111
    for k, v in kw.items():
        setattr(p, k, v)
    return p.finalize()


WORKLOADS = {
    "hex32_plain": dict(n=32, defect=4, ME=False, rot111=False, steps=500, B0=0.1),
    "hex128_me": dict(n=128, defect=16, ME=True, rot111=True, steps=500, B0=0.1),
    "hex64_me": dict(n=64, defect=8, ME=True, rot111=True, steps=500, B0=0.1),
    "hex256_plain": dict(n=256, defect=32, ME=False, rot111=True, steps=200, B0=0.1),
    "hex192_me": dict(n=192, defect=24, ME=True, rot111=True, steps=200, B0=0.1),
}


TET_WORKLOADS = {
    # 96^3 cube of Kuhn tets (5.3 M tets), interior nodes jittered +-0.2 h, rotated ellipsoidal defect
    "tet96_me": dict(n=96, jitter=0.2, axes=(0.15, 0.10, 0.08), ME=True, rot111=True, steps=300, B0=0.1, seed=96),
    "tet32_me": dict(n=32, jitter=0.2, axes=(0.15, 0.10, 0.08), ME=True, rot111=True, steps=300, B0=0.1, seed=32),
}


def seeded_rotation(seed):
    """A proper rotation matrix from the QR factors of a seeded normal matrix."""
    rng = np.random.default_rng(seed)
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q @ np.diag(np.sign(np.diag(r)))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def tet_workload(w):
    """(params, mesh) of a Kuhn-tet cube: edge n (h = 1, the reference's length unit), the defect's
    semi-axes a fraction of the edge, centred at the box centre, with a seeded rotation."""
    from .mesh.grids import TetraGrid, kuhn_tet_cube
    from .utils.defect_shapes import get_defect_shape_function
    n = w["n"]
    coords, tets = kuhn_tet_cube(n, jitter=w["jitter"], seed=w["seed"])
    axes = tuple(float(f) * n for f in w["axes"])
    R = seeded_rotation(w["seed"] + 1)
    p = SimParams(**MAGNETIC)
    if w["ME"]:
        for k, v in ELASTIC.items():
            setattr(p, k, v)
    p.grid_type = "Tet"
    p.ME = w["ME"]
    p.rot111 = w["rot111"]
    p.defect_shape = "RotatedEllipsoid"
    p.defect_parameters = axes
    p.defect_rotation = R.tolist()
    p = p.finalize()
    mesh = TetraGrid(coords=coords, tets=tets,
                     defect_shape=get_defect_shape_function("RotatedEllipsoid", (axes, R)))
    return p, mesh


def workload(name, **overrides):
    """(params, workload dict); tet workloads carry their in-memory mesh as w["mesh"]."""
    if name in TET_WORKLOADS:
        w = dict(TET_WORKLOADS[name])
        w.update(overrides)
        p, w["mesh"] = tet_workload(w)
        w["defect"] = "ellipsoid %s" % (tuple(round(a * w["n"], 2) for a in w["axes"]),)
        return p, w
    w = dict(WORKLOADS[name])
    w.update(overrides)
    p = hex_params(w["n"], w["defect"], w["ME"], w["rot111"])
    return p, w


def sweep_field(p: SimParams, s: int, steps: int, B0: float):
    """Applied field (normalised) at step s of a linear +B0 -> -B0 tesla sweep along x."""
    frac = s / (steps - 1) if steps > 1 else 0.0
    H1 = (B0 - 2.0 * B0 * frac) / MU0
    return (H1 / p.ms, 0.0, 0.0)


def seeded_m0(n_dof, defect_dofs, seed=1234, sigma=1e-3):
    rng = np.random.default_rng(seed)
    m = np.array([1.0, 0.0, 0.0])[None, :] + rng.normal(0.0, sigma, size=(n_dof, 3))
    m /= np.linalg.norm(m, axis=1, keepdims=True)
    m[np.asarray(defect_dofs, dtype=np.int64)] = 0.0
    return m
