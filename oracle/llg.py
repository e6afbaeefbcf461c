"""One Gauss-Seidel-projection LLG step and the drivers around it (oracle).

Restates cupymag/core/Micromagnetics.py:110-307 line by line in NumPy/SciPy:

* ME block (:114-164): eigenstrain E0(m) (final_assembly.py:208-266), rotated
  by M^T when rot111; b_el = F_el E0; elastic CG; strain from u
  (compute_derivatives.py:60-125); mean removal; macroscopic strain E_bar from
  the magnetostriction of <m> plus S sigma (sigma_matrices.py:25-46);
  rotation by M^{-T}.
* demag (:166-172): b = -(Fx m~x + Fy m~y + Fz m~z), b[0] = 0, CG, H~ = -F U,
  H_bar = -N <m>.
* effective field (:175-211) and the Gauss-Seidel chain (:213-290).
* renormalise, defect zero, sumsq, warm-start rule (:292-301), averages
  (:306-307).
"""
import math

import numpy as np

from .cg import solve_cg

INV_SQRT2 = 1.0 / math.sqrt(2.0)
INV_SQRT3 = 1.0 / math.sqrt(3.0)
INV_SQRT6 = 1.0 / math.sqrt(6.0)


def R_matrix():
    """x -> [111] rotation (cupymag/utils/rot_111_matrices.py:21-59)."""
    return np.array([[INV_SQRT3, INV_SQRT3, INV_SQRT3],
                     [-INV_SQRT2, INV_SQRT2, 0.0],
                     [-INV_SQRT6, -INV_SQRT6, 2 * INV_SQRT6]])


def M_matrix():
    """Voigt rotation for the [111] frame (rot_111_matrices.py:62-103)."""
    s2, s3 = math.sqrt(2.0), math.sqrt(3.0)
    return np.array([
        [1 / 3, 1 / 3, 1 / 3, 2 / 3, 2 / 3, 2 / 3],
        [1 / 2, 1 / 2, 0.0, 0.0, 0.0, -1.0],
        [1 / 6, 1 / 6, 2 / 3, -2 / 3, -2 / 3, 1 / 3],
        [s3 / 6, -s3 / 6, 0.0, s3 / 3, -s3 / 3, 0.0],
        [-s2 / 6, -s2 / 6, s2 / 3, s2 / 6, s2 / 6, -s2 / 3],
        [-INV_SQRT6, INV_SQRT6, 0.0, INV_SQRT6, -INV_SQRT6, 0.0]])


def ebar_sigma(p):
    S = np.zeros((6, 6))
    S[0, 0] = S[1, 1] = S[2, 2] = p.s11
    S[3, 3] = S[4, 4] = S[5, 5] = p.s44
    S[0, 1] = S[0, 2] = S[1, 0] = S[1, 2] = S[2, 0] = S[2, 1] = p.s12
    return S @ np.array(p.sigma, dtype=np.float64)


def build_E0(lam100, lam111, m):
    n = m.shape[0]
    E0 = np.zeros(6 * n)
    mx, my, mz = m[:, 0], m[:, 1], m[:, 2]
    E0[0::6] = 1.5 * lam100 * (mx * mx - 1.0 / 3.0)
    E0[1::6] = 1.5 * lam100 * (my * my - 1.0 / 3.0)
    E0[2::6] = 1.5 * lam100 * (mz * mz - 1.0 / 3.0)
    E0[3::6] = 2.0 * (1.5 * lam111 * (mx * my))
    E0[4::6] = 2.0 * (1.5 * lam111 * (my * mz))
    E0[5::6] = 2.0 * (1.5 * lam111 * (mx * mz))
    return E0


def strain_from_u(ops, n, u, R=None):
    Dx, Dy, Dz = ops["Fx"], ops["Fy"], ops["Fz"]
    ux, uy, uz = u[:n], u[n:2 * n], u[2 * n:]
    if R is None:
        return np.stack([Dx @ ux, Dy @ uy, Dz @ uz, Dy @ ux + Dx @ uy, Dz @ uy + Dy @ uz, Dz @ ux + Dx @ uz],
                        axis=-1)
    dxx, dyx, dzx = Dx @ ux, Dy @ ux, Dz @ ux
    dxy, dyy, dzy = Dx @ uy, Dy @ uy, Dz @ uy
    dxz, dyz, dzz = Dx @ uz, Dy @ uz, Dz @ uz
    E11 = R[0, 0] * dxx + R[1, 0] * dyx + R[2, 0] * dzx
    E22 = R[0, 1] * dxy + R[1, 1] * dyy + R[2, 1] * dzy
    E33 = R[0, 2] * dxz + R[1, 2] * dyz + R[2, 2] * dzz
    E12 = (R[0, 1] * dxx + R[1, 1] * dyx + R[2, 1] * dzx) + (R[0, 0] * dxy + R[1, 0] * dyy + R[2, 0] * dzy)
    E23 = (R[0, 2] * dxy + R[1, 2] * dyy + R[2, 2] * dzy) + (R[0, 1] * dxz + R[1, 1] * dyz + R[2, 1] * dzz)
    E13 = (R[0, 2] * dxx + R[1, 2] * dyx + R[2, 2] * dzx) + (R[0, 0] * dxz + R[1, 0] * dyz + R[2, 0] * dzz)
    return np.stack([E11, E22, E33, E12, E23, E13], axis=-1)


def _aniso_me(K1, C1, C2, C3, lam100, mm, E):
    """First derivatives of anisotropy + magnetoelastic energy (Micromagnetics.py:181-206)."""
    m1, m2, m3 = mm[:, 0], mm[:, 1], mm[:, 2]
    s1, s2, s3 = m1 * m1, m2 * m2, m3 * m3
    v1 = (-2.0 * K1 * m1 * (s2 + s3) - 2.0 * C1 * m1 * (s2 + s3) - 2.0 * C2 * (E[:, 0] - lam100) * m1
          - C3 * (E[:, 3] * m2 + E[:, 5] * m3))
    v2 = (-2.0 * K1 * m2 * (s3 + s1) - 2.0 * C1 * m2 * (s3 + s1) - 2.0 * C2 * (E[:, 1] - lam100) * m2
          - C3 * (E[:, 4] * m3 + E[:, 3] * m1))
    v3 = (-2.0 * K1 * m3 * (s1 + s2) - 2.0 * C1 * m3 * (s1 + s2) - 2.0 * C2 * (E[:, 2] - lam100) * m3
          - C3 * (E[:, 5] * m1 + E[:, 4] * m2))
    return v1, v2, v3


def effective_field(p, m, E, Hbar, Ht, Hext, R=None):
    """f1..f3 of Micromagnetics.py:175-211 (rot111 variant when R is given)."""
    C1, C2, C3 = p.step_elasC
    if R is None:
        # same association order as Micromagnetics.py:181-189
        K1, lam = p.K1, p.lambda100
        m1, m2, m3 = m[:, 0], m[:, 1], m[:, 2]
        s1, s2, s3 = m1 * m1, m2 * m2, m3 * m3
        f1 = (-2.0 * K1 * m1 * (s2 + s3) + 0.5 * Hbar[0] + 0.5 * Ht[0] + Hext[0]
              - 2.0 * C1 * m1 * (s2 + s3) - 2.0 * C2 * (E[:, 0] - lam) * m1 - C3 * (E[:, 3] * m2 + E[:, 5] * m3))
        f2 = (-2.0 * K1 * m2 * (s3 + s1) + 0.5 * Hbar[1] + 0.5 * Ht[1] + Hext[1]
              - 2.0 * C1 * m2 * (s3 + s1) - 2.0 * C2 * (E[:, 1] - lam) * m2 - C3 * (E[:, 4] * m3 + E[:, 3] * m1))
        f3 = (-2.0 * K1 * m3 * (s1 + s2) + 0.5 * Hbar[2] + 0.5 * Ht[2] + Hext[2]
              - 2.0 * C1 * m3 * (s1 + s2) - 2.0 * C2 * (E[:, 2] - lam) * m3 - C3 * (E[:, 5] * m1 + E[:, 4] * m2))
        return f1, f2, f3
    else:
        m100 = m @ R
        v = np.stack(_aniso_me(p.K1, C1, C2, C3, p.lambda100, m100, E), axis=-1) @ R.T
        v1, v2, v3 = v[:, 0], v[:, 1], v[:, 2]
    f1 = v1 + 0.5 * Hbar[0] + 0.5 * Ht[0] + Hext[0]
    f2 = v2 + 0.5 * Hbar[1] + 0.5 * Ht[1] + Hext[1]
    f3 = v3 + 0.5 * Hbar[2] + 0.5 * Ht[2] + Hext[2]
    return f1, f2, f3


class LLGState:
    def __init__(self, m, avg):
        self.m = m.copy()
        self.m_prev = m.copy()
        self.avg_m = avg(self.m)
        self.m_tilde = self.m - self.avg_m
        self.use_init = False
        self.x = {}
        self.E = None
        self.Ht = None
        self.sumsq = np.inf
        self.iters = []


def llg_step(S, ops, Avg, p, Hext, defect, maxiter=None, dot=None):
    """Advance S by one GSPM step at applied field Hext (nondimensional).

    dot: the CG inner product (None: np.dot, the restatement's own order)."""
    n = S.m.shape[0]
    tol = p.tol
    maxiter = p.maxiter if maxiter is None else maxiter
    R = R_matrix() if p.rot111 else None
    M = M_matrix() if p.rot111 else None
    m = S.m
    ui = S.use_init
    rec = S.iters
    X = S.x

    def cg(A, b, key):
        x = solve_cg(A, b, x0=X.get(key), tol=tol, maxiter=maxiter, use_init=ui, system=key, record=rec, dot=dot)
        X[key] = x
        return x

    m100 = m @ R if p.rot111 else None
    if p.ME:
        if p.rot111:
            E0 = (build_E0(p.lambda100, p.lambda111, m100).reshape(n, 6) @ M.T).reshape(6 * n)
        else:
            E0 = build_E0(p.lambda100, p.lambda111, m)
        b_el = ops["F_el"] @ E0
        u = cg(ops["A_el"], b_el, "elasticity")
        E = strain_from_u(ops, n, u, R)
        E = E - Avg(E)
        Es = ebar_sigma(p)
        am = Avg(m100) if p.rot111 else S.avg_m
        Eb = np.array([1.5 * p.lambda100 * (am[0] ** 2 - 1 / 3) + Es[0],
                       1.5 * p.lambda100 * (am[1] ** 2 - 1 / 3) + Es[1],
                       1.5 * p.lambda100 * (am[2] ** 2 - 1 / 3) + Es[2],
                       3.0 * p.lambda111 * am[0] * am[1] + Es[3],
                       3.0 * p.lambda111 * am[1] * am[2] + Es[4],
                       3.0 * p.lambda111 * am[0] * am[2] + Es[5]])
        if p.rot111:
            Eb = M @ Eb
        E = E + Eb[None, :]
        if p.rot111:
            E = E @ np.linalg.inv(M).T
    else:
        E = np.zeros((n, 6))

    mt = S.m_tilde
    b_demag = -(ops["Fx"] @ mt[:, 0] + ops["Fy"] @ mt[:, 1] + ops["Fz"] @ mt[:, 2])
    b_demag[0] = 0.0
    U = cg(ops["A_demag"], b_demag, "demag")
    Ht = (-(ops["Fx"] @ U), -(ops["Fy"] @ U), -(ops["Fz"] @ U))
    Hbar = (-p.N_x * S.avg_m[0], -p.N_y * S.avg_m[1], -p.N_z * S.avg_m[2])

    f1, f2, f3 = effective_field(p, m, E, Hbar, Ht, Hext, R)
    dt = p.dt
    F1, A1, A2 = ops["F1"], ops["A1"], ops["A2"]
    g1n = cg(A1, F1 @ (f1 * dt + m[:, 0]), "g1n")
    g2n = cg(A1, F1 @ (f2 * dt + m[:, 1]), "g2n")
    g3n = cg(A1, F1 @ (f3 * dt + m[:, 2]), "g3n")
    m1s = m[:, 0] + g2n * m[:, 2] - g3n * m[:, 1]
    g1s = cg(A1, F1 @ (f1 * dt + m1s), "g1star")
    m2s = m[:, 1] + g3n * m1s - g1s * m[:, 2]
    g2s = cg(A1, F1 @ (f2 * dt + m2s), "g2star")
    m3s = m[:, 2] + g1s * m2s - g2s * m1s

    dt2 = dt * p.alpha_damp
    ms = np.stack([m1s, m2s, m3s], axis=-1)
    h1, h2, h3 = effective_field(p, ms, E, Hbar, Ht, Hext, R)
    mss1 = cg(A2, F1 @ (h1 * dt2 + m1s), "m1starstar")
    mss2 = cg(A2, F1 @ (h2 * dt2 + m2s), "m2starstar")
    mss3 = cg(A2, F1 @ (h3 * dt2 + m3s), "m3starstar")

    mag = np.sqrt(mss1 ** 2 + mss2 ** 2 + mss3 ** 2)
    small = np.abs(mag) < 1e-14
    safe = np.where(small, 1.0, mag)
    mnew = np.stack([np.where(small, 0.0, mss1 / safe), np.where(small, 0.0, mss2 / safe),
                     np.where(small, 0.0, mss3 / safe)], axis=-1)
    mnew[defect, :] = 0.0
    sumsq = float(np.sum((mnew - S.m_prev) ** 2))
    LLG_accuracy = n * p.LLG_accuracy_factor
    S.use_init = bool(sumsq < p.use_init_factor * LLG_accuracy)
    S.m = mnew
    S.m_prev = mnew.copy()
    S.sumsq = sumsq
    S.avg_m = Avg(mnew)
    S.m_tilde = mnew - S.avg_m
    S.E = E
    S.Ht = Ht
    return S


def fixed_sweep_fields(p, steps, B0):
    """Applied field per step for a linear sweep +B0 -> -B0 tesla along x.

    H1_s = (B0 - 2 B0 s/(S-1)) / MU0 in A/m, normalised by Ms.
    """
    from_mu0 = 1.25663706127e-6
    out = []
    for s in range(steps):
        frac = s / (steps - 1) if steps > 1 else 0.0
        H1 = (B0 - 2.0 * B0 * frac) / from_mu0
        out.append((H1 / p.ms, 0.0, 0.0))
    return out


def run_driver(p, ops, Avg, defect, m0, max_steps=100000, dot=None):
    """The reference's convergence-driven field sweep (Micromagnetics.py:76-347).

    Returns the hysteresis rows [Hext1, Hext2, Hext3, <m1>, <m2>, <m3>] (H in
    A/m) written at every convergence/save event and at the end, and the final m.
    """
    n = m0.shape[0]
    S = LLGState(m0, Avg)
    llg_min_step = 10 if p.ME else 100
    LLG_accuracy = n * p.LLG_accuracy_factor
    Hext = list(p.Hext)
    dH = list(p.dHext)
    stop = np.asarray(p.stop_direction, dtype=np.float64)
    rows = []
    nstep = 0
    total = 0
    while S.avg_m @ stop > p.stop_value and total < max_steps:
        nstep += 1
        total += 1
        llg_step(S, ops, Avg, p, tuple(Hext), defect, dot=dot)
        conv = S.sumsq < LLG_accuracy and nstep > llg_min_step
        if conv or nstep % p.save_frequency == 0:
            rows.append([float(f"{Hext[0] * p.ms:.1f}"), float(f"{Hext[1] * p.ms:.1f}"),
                         float(f"{Hext[2] * p.ms:.1f}"), *S.avg_m])
        if conv:
            Hext = [h - d for h, d in zip(Hext, dH)]
            nstep = 0
    rows.append([float(f"{Hext[0] * p.ms:.1f}"), float(f"{Hext[1] * p.ms:.1f}"), float(f"{Hext[2] * p.ms:.1f}"),
                 *S.avg_m])
    return np.array(rows), S.m, total
