"""The Gauss-Seidel-projection LLG step on the GPU.

Restates the step body of cupymag/core/Micromagnetics.py:110-307 (which in
the reference exists only inline in ``main``) as device kernels launched on
one CUDA stream, with no host synchronisation inside a step:

1. magnetoelastic equilibrium (:114-164): eigenstrain E0(m) -> b_el = F_el E0
   -> CG on A_el -> strain E from u -> E - <E> + E_bar -> rotate;
2. demag (:166-172): b = -F.(m - <m>), b[0] = 0 -> CG on A_demag -> H~ = -F U;
3. field f(m) and t = f dt + m (:175-215); b = F1 t for the three components,
   one 3-right-hand-side CG on A1 -> (g1n, g2n, g3n) (:217-223);
4. the star chain m1*, g1* (CG on A1), m2*, g2* (CG on A1), m3* (:225-237);
5. field at m* with dt2 = dt alpha, b = F1 t, one 3-RHS CG on A2 -> m** (:239-290);
6. renormalise, zero the defect, sumsq, the warm-start flag and <m>
   (:292-307), all in one kernel.

The warm-start decision ``use_init = sumsq < initial_factor * n * accuracy``
(:88,299-300) stays on the device: step k+1's solvers read the flag written
by step k, so steps can be queued (or captured in a CUDA graph) back to back.
Solver results (status, iterations, residuals) land in a device array that
``check()`` reads once per step; a solve that did not converge raises the
reference's RuntimeError text.

Public entry points (the north-star "physics" functions the reference keeps
inline): ``effective_field``, ``magnetoelastic_strain``, ``demag_field``,
``gs_projection_step`` and ``LLGSolver.step``.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np
import torch

from .. import _native as N
from ..solvers.linear_solvers import CGSolver, ResidualCarry, decode_info, new_info, raise_for
from ..utils.rot_111_matrices import get_M_matrix, get_R_matrix
from ..utils.sigma_matrices import get_Ebar_sigma

# order of the solves recorded per step (same order as the reference's solve_cg calls)
SOLVE_NAMES = ["elasticity", "demag", "Gauss-Seidel g1n/g2n/g3n", "Gauss-Seidel g1star", "Gauss-Seidel g2star",
               "Gauss-Seidel m1starstar/m2starstar/m3starstar"]

# Reliable-update factor of the FP32 solver per solve (a true residual whenever the FP32 residual has
# fallen by this factor: FP64, or double-float for A1/A2 where its proven error bound allows).  Measured on GB300 at 64^3-128^3: the ill-conditioned
# elasticity solve converges in the fewest iterations with 0.1 (smaller factors add 25-40 %
# iterations); the Gauss-Seidel solves (A1, A2; ~30-55 iterations) converge in the same
# iterations down to 1e-5, so fewer FP64 products win: at 128^3 (cold, 1 and 3 right-hand sides)
# 1e-4 takes three FP64 residuals, 1e-5 two at the same iteration counts (7-10 % faster), 1e-6
# adds an iteration; demag is best near 1e-3.
INNER_TOL = [0.1, 1e-3, 1e-5, 1e-5, 1e-5, 1e-5]

# Solves that the precision form runs with the FFT solver on stencil operators: elasticity and demag,
# whose operators are circulant apart from the anchor at node 0, so each FP64 refinement step solves
# them exactly with one FFT apply (two steps per solve at 128^3).  The Gauss-Seidel operators A1/A2 carry
# the defect rows and columns; plain FP32 CG needs only 20-55 iterations there, and the circulant inverse
# as a preconditioner does not lower that.  FFT_INNER_TOL is the inner drop of the preconditioned-CG form,
# used where an operator has no single anchor.
FFT_SLOTS = (0, 1)
FFT_INNER_TOL = 1e-4

# NVTX ranges around the stages of a step (magnetoelastic, demag, Gauss-Seidel projection) when
# CPM_NVTX=1, so a profiler's timeline shows where a step's time goes; off by default (no calls).
NVTX = os.environ.get("CPM_NVTX") == "1"


def _range_push(name):
    if NVTX:
        torch.cuda.nvtx.range_push(name)


def _range_pop():
    if NVTX:
        torch.cuda.nvtx.range_pop()


class LLGSolver:
    """Device-resident state and operators of one LLG run."""

    def __init__(self, sim_ops, params, precision="DP", device=None, ops=None, operators="csr", info=None,
                 precond="auto"):
        """precond: "fft" runs the elastic and demag solves of the precision form with the FFT solver
        (stencil operators only: the exact solve of the anchored operator inside FP64 refinement), None
        runs every solve as plain CG; "auto" is "fft" for the precision form on stencil operators."""
        self.p = params
        self.precision = "DP" if precision == "DP" else "IR"
        if precond == "auto":
            precond = "fft" if (self.precision == "IR" and operators == "stencil") else None
        if precond not in (None, "fft"):
            raise ValueError(f"unknown preconditioner {precond!r}")
        self.precond = precond
        self.dev = device or sim_ops.device
        dev = self.dev
        self.n = n = sim_ops.n_dof
        self.operators = operators
        if operators == "stencil":
            # matrix-free forms of every operator of the step (structured hex grids): the solved
            # operators, F1, the derivative matrices Fx, Fy, Fz and F_el; no CSR matrix is resident
            if ops is None:
                ops = sim_ops.stencil_step_operators()
            A_demag, Fx, Fy, Fz, Deriv, A1, A2, F1, A_el, F_el, Avg = ops
            if not hasattr(A_demag, "ncomp"):
                raise ValueError("operators='stencil' needs matrix-free operators in ops")
            if F_el is None and params.ME:
                raise ValueError("magnetoelastic run without F_el")
        elif ops is None:
            A_demag, Fx, Fy, Fz, Deriv = sim_ops.csr_demag_and_deriv()
            A1, A2, F1 = sim_ops.csr_GS()
            A_el, F_el = sim_ops.csr_elasticity()
            Avg = sim_ops.volume_average()
        else:
            A_demag, Fx, Fy, Fz, Deriv, A1, A2, F1, A_el, F_el, Avg = ops
        self.A_demag, self.Fx, self.Fy, self.Fz, self.Deriv = A_demag, Fx, Fy, Fz, Deriv
        self.A1, self.A2, self.F1, self.A_el, self.F_el, self.Avg = A1, A2, F1, A_el, F_el, Avg
        if self.precision == "IR":
            for A in (A_demag, A1, A2, A_el):
                if A is not None:
                    A.ensure_fp32()
        self.ME = bool(params.ME) and A_el is not None
        self.rot = bool(params.rot111)
        self.solver = CGSolver(dev)
        f64 = dict(dtype=torch.float64, device=dev)
        z = lambda *s: torch.zeros(*s, **f64)  # noqa: E731
        self.m, self.m_prev, self.mss, self.mstar = z(n, 3), z(n, 3), z(n, 3), z(n, 3)
        self.avg_m, self.avg_m100, self.avgE = z(3), z(3), z(6)
        self.sumsq = torch.full((1,), math.inf, **f64)
        self.use_init = torch.zeros(1, dtype=torch.int32, device=dev)
        self.U, self.g, self.g1s, self.g2s = z(n), z(n, 3), z(n), z(n)
        self.Ht, self.f, self.t, self.b3 = z(n, 3), z(n, 3), z(n, 3), z(n, 3)
        self.b1, self.t1, self.bdemag = z(n), z(n), z(n)
        if self.ME:
            self.u, self.E, self.E0, self.b_el = z(3 * n), z(n, 6), z(6 * n), z(3 * n)
        else:
            self.u = self.E = self.E0 = self.b_el = None
        if info is None:
            info = new_info(len(SOLVE_NAMES), dev)
        elif tuple(info.shape) != (len(SOLVE_NAMES), N.CG_INFO_BYTES):
            raise ValueError(f"info must be a ({len(SOLVE_NAMES)}, {N.CG_INFO_BYTES}) uint8 device tensor")
        self.info = info
        self.hsched = self.hstep = self.hist = None
        mask = np.zeros(n, dtype=np.uint8)
        mask[np.asarray(sim_ops.DefDOF, dtype=np.int64)] = 1
        self.defect = torch.as_tensor(mask, device=dev)
        self.scratch = torch.zeros(N.lib().cpm_volavg_scratch_doubles(6), **f64)
        self.R9 = get_R_matrix().reshape(-1)
        self.R9_dev = torch.as_tensor(self.R9, **f64)
        M = get_M_matrix()
        self.M36_dev = torch.as_tensor(M.reshape(-1), **f64)
        self.MinvT36_dev = torch.as_tensor(np.linalg.inv(M).T.reshape(-1).copy(), **f64)
        self.Es_dev = torch.as_tensor(get_Ebar_sigma(params), **f64)
        # residual carries of the FFT solves (elasticity: 3n unknowns, demag: n), keyed by slot
        self.carry = {}
        if self.precond == "fft" and self.precision == "IR":
            self.carry[1] = ResidualCarry(n, dev)
            if self.ME:
                self.carry[0] = ResidualCarry(3 * n, dev)
        self.thresh = params.use_init_factor * (n * params.LLG_accuracy_factor)
        self.nstep = 0
        self.launches = 0          # kernels this solver has launched (C-ABI calls that start one kernel)

    # ------------------------------------------------------------------ state
    def set_magnetization(self, m0):
        m0 = torch.as_tensor(m0, dtype=torch.float64).reshape(self.n, 3)
        if self.hstep is not None:
            self.hstep.zero_()
        self.m.copy_(m0, non_blocking=True)
        self.m_prev.copy_(self.m)
        self.Avg.average_into(self.m, self.avg_m)
        self.use_init.zero_()
        for c in self.carry.values():
            c.invalidate()
        self.sumsq.fill_(math.inf)
        self.nstep = 0

    def set_field_schedule(self, fields):
        """Drive the applied field from a device schedule (steps, 3), normalised by Ms.

        Step s then uses fields[s] read on the device from a step counter that
        the end of each step advances, so a step captured once in a CUDA graph
        follows the sweep when replayed; the Hext argument of step() is then
        ignored.  Each step also records (<m>, sumsq) into ``hist`` (steps, 4)."""
        f = torch.as_tensor(np.asarray(fields, dtype=np.float64).reshape(-1, 3), device=self.dev)
        self.hsched = f.contiguous()
        self.hstep = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.hist = torch.zeros((f.shape[0], 4), dtype=torch.float64, device=self.dev)

    # ------------------------------------------------------------------ checkpoint / resume
    def _state_tensors(self):
        """Every device tensor that carries over from one step to the next: m, m_prev, <m>, sumsq,
        the warm-start flag, the previous solutions the warm-started solves start from (U, the g's,
        m**, and u with magnetoelastic coupling), the FFT solves' residual carries and the field-schedule
        position."""
        t = {"m": self.m, "m_prev": self.m_prev, "avg_m": self.avg_m, "sumsq": self.sumsq, "use_init": self.use_init,
             "U": self.U, "g": self.g, "g1s": self.g1s, "g2s": self.g2s, "mss": self.mss}
        if self.ME:
            t["u"] = self.u
        for k, c in self.carry.items():
            t.update({f"carry{k}_b": c.b, f"carry{k}_t": c.t, f"carry{k}_valid": c.valid})
        if self.hsched is not None:
            t.update(hsched=self.hsched, hstep=self.hstep, hist=self.hist)
        return t

    def save_state(self, path):
        """Write the run's state (.npz) so that load_state + further steps reproduce an uninterrupted run
        bit for bit (the reference restarts from m alone, magnetization_io.py:80-124)."""
        arrays = {k: v.detach().cpu().numpy() for k, v in self._state_tensors().items()}
        np.savez(path, nstep=np.int64(self.nstep), n=np.int64(self.n), ME=np.int8(self.ME),
                 precision=np.str_(self.precision), operators=np.str_(self.operators), **arrays)

    def load_state(self, path):
        """Restore a save_state checkpoint.  The checkpoint must come from a run of the same size,
        coupling, precision form and operator form (a run's warm-start vectors and iterates depend on
        all four); a field schedule already set on this solver must have the checkpoint's length."""
        d = np.load(path)
        if int(d["n"]) != self.n or bool(d["ME"]) != self.ME:
            raise ValueError(f"checkpoint of a different run (n={int(d['n'])}, ME={bool(d['ME'])})")
        for key, mine in (("precision", self.precision), ("operators", self.operators)):
            if key not in d:
                raise ValueError(f"checkpoint lacks {key}")
            if str(d[key]) != str(mine):
                raise ValueError(f"checkpoint of a run with {key}={str(d[key])!r}, this solver has {mine!r}")
        if "hsched" in d and self.hsched is not None and tuple(d["hsched"].shape) != tuple(self.hsched.shape):
            raise ValueError(f"checkpoint field schedule has {d['hsched'].shape[0]} steps, this solver's has "
                             f"{self.hsched.shape[0]}")
        if "hsched" in d and self.hsched is None:
            self.set_field_schedule(d["hsched"])
        for k, t in self._state_tensors().items():
            if k not in d:
                if k.startswith("carry"):
                    continue  # a checkpoint without carries: the next FFT solves start from FP64 residuals
                raise ValueError(f"checkpoint lacks {k}")
            t.copy_(torch.as_tensor(d[k], device=self.dev))
        for k, c in self.carry.items():
            if f"carry{k}_valid" not in d:
                c.invalidate()
        self.nstep = int(d["nstep"])

    # ------------------------------------------------------------------ building blocks
    def _field_params(self, Hext):
        P = N.FieldParams()
        C1, C2, C3 = self.p.step_elasC
        P.K1, P.elasC1, P.elasC2, P.elasC3, P.lambda100 = self.p.K1, C1, C2, C3, self.p.lambda100
        P.Nd[:] = (self.p.N_x, self.p.N_y, self.p.N_z)
        P.Hext[:] = (0.0, 0.0, 0.0) if Hext is None else tuple(float(h) for h in Hext)
        P.R[:] = tuple(self.R9)
        P.rot111 = 1 if self.rot else 0
        P.has_E = 1 if self.ME else 0
        if self.hsched is not None:
            P.hext_sched = self.hsched.data_ptr()
            P.hext_step = self.hstep.data_ptr()
        return P

    def _cg(self, A, b, x, k):
        self.launches += 1
        fft = self.precond == "fft" and k in FFT_SLOTS
        self.solver.launch(A, b, x, self.info[k], tol=self.p.tol, maxiter=self.p.maxiter,
                           use_init_dev=self.use_init, precision=self.precision,
                           inner_tol=FFT_INNER_TOL if fft else INNER_TOL[k], precond="fft" if fft else None,
                           carry=self.carry.get(k) if fft else None)

    def cg_request(self, A, b, x, k):
        """A solve of this step, for an executor that batches solves of several runs."""
        return CGRequest(self, A, b, x, k)

    @staticmethod
    def _run(gen):
        for req in gen:
            req.execute()

    def magnetoelastic_strain(self):
        """E from mechanical equilibrium at the current m (Micromagnetics.py:114-164)."""
        self._run(self._me_gen())
        return self.E

    def _me_gen(self):
        L, s = N.lib(), N.stream_ptr()
        n, p = self.n, self.p
        R9 = self.R9_dev.data_ptr() if self.rot else None
        M36 = self.M36_dev.data_ptr() if self.rot else None
        N.check(L.cpm_build_E0(n, self.m.data_ptr(), p.lambda100, p.lambda111, R9, M36, self.E0.data_ptr(), s),
                "cpm_build_E0")
        self.F_el.spmv(self.E0, out=self.b_el)
        self.launches += 5 + (1 if self.rot else 0)
        yield self.cg_request(self.A_el, self.b_el, self.u, 0)
        self.Deriv.strain_into(self.u, self.E, self.R9_dev if self.rot else None)
        self.Avg.average_into(self.E, self.avgE)
        if self.rot:
            self.Avg.average_into(self.m, self.avg_m100, R9=self.R9_dev)
            am = self.avg_m100
        else:
            am = self.avg_m
        N.check(L.cpm_strain_finalize(n, self.E.data_ptr(), self.avgE.data_ptr(), am.data_ptr(), p.lambda100,
                                      p.lambda111, self.Es_dev.data_ptr(), self.M36_dev.data_ptr(),
                                      self.MinvT36_dev.data_ptr(), 1 if self.rot else 0, s), "cpm_strain_finalize")

    def demag_field(self):
        """H~ = -F U with U from the pinned demag Poisson solve (Micromagnetics.py:166-171)."""
        self._run(self._demag_gen())
        return self.Ht

    def _demag_gen(self):
        self.Deriv.demag_rhs_into(self.m, self.avg_m, self.bdemag, pin=0)
        self.launches += 2
        yield self.cg_request(self.A_demag, self.bdemag, self.U, 1)
        self.Deriv.hd_into(self.U, self.Ht)

    def effective_field(self, mm, dt, Hext, f_out=None, t_out=None):
        """f(mm) and t = f dt + mm (Micromagnetics.py:175-215 / :239-278)."""
        t_out = self.t if t_out is None else t_out
        self.launches += 1
        N.check(N.lib().cpm_llg_field(C.byref(self._field_params(Hext)), self.n, mm.data_ptr(),
                                      self.E.data_ptr() if self.ME else None, self.Ht.data_ptr(),
                                      self.avg_m.data_ptr(), float(dt), None if f_out is None else f_out.data_ptr(),
                                      t_out.data_ptr(), N.stream_ptr()), "cpm_llg_field")
        return t_out

    def gs_projection_step(self, Hext):
        """Gauss-Seidel projection with the current fields, then renormalisation (:213-307)."""
        self._run(self._gs_gen(Hext))

    def _gs_gen(self, Hext):
        L, s, n, p = N.lib(), N.stream_ptr(), self.n, self.p
        dt = p.dt
        self.effective_field(self.m, dt, Hext, f_out=self.f, t_out=self.t)
        self.launches += 8  # 4 SpMV, 3 star updates, 1 renormalisation (fields and CGs count themselves)
        self.F1.spmv(self.t, out=self.b3)
        yield self.cg_request(self.A1, self.b3, self.g, 2)
        mp, gp = self.m.data_ptr(), self.g.data_ptr()
        N.check(L.cpm_gs_star(1, n, mp, gp, None, None, self.f.data_ptr(), dt, self.mstar.data_ptr(),
                              self.t1.data_ptr(), s), "cpm_gs_star")
        self.F1.spmv(self.t1, out=self.b1)
        yield self.cg_request(self.A1, self.b1, self.g1s, 3)
        N.check(L.cpm_gs_star(2, n, mp, gp, self.g1s.data_ptr(), None, self.f.data_ptr(), dt,
                              self.mstar.data_ptr(), self.t1.data_ptr(), s), "cpm_gs_star")
        self.F1.spmv(self.t1, out=self.b1)
        yield self.cg_request(self.A1, self.b1, self.g2s, 4)
        N.check(L.cpm_gs_star(3, n, mp, gp, self.g1s.data_ptr(), self.g2s.data_ptr(), None, dt,
                              self.mstar.data_ptr(), None, s), "cpm_gs_star")
        self.effective_field(self.mstar, dt * p.alpha_damp, Hext, t_out=self.t)
        self.F1.spmv(self.t, out=self.b3)
        yield self.cg_request(self.A2, self.b3, self.mss, 5)
        w, V = self.Avg.weights()
        N.check(L.cpm_renorm_sumsq(n, self.mss.data_ptr(), self.defect.data_ptr(), self.m.data_ptr(),
                                   self.m_prev.data_ptr(), w.data_ptr(), V, self.thresh, self.sumsq.data_ptr(),
                                   self.avg_m.data_ptr(), self.use_init.data_ptr(), self.scratch.data_ptr(), s),
                "cpm_renorm_sumsq")
        if self.hsched is not None:
            self.launches += 1
            N.check(L.cpm_record_step(self.avg_m.data_ptr(), self.sumsq.data_ptr(), self.hist.data_ptr(),
                                      self.hstep.data_ptr(), self.hist.shape[0], s), "cpm_record_step")

    def step(self, Hext):
        """One GSPM step at applied field Hext (normalised by Ms); asynchronous."""
        self._run(self.step_gen(Hext))

    def step_gen(self, Hext):
        """The step as a generator that yields each linear solve (CGRequest) before it is needed.

        The caller executes every yielded request before resuming; a batching
        executor can collect the requests of several runs and solve them in
        one launch."""
        if self.ME:
            _range_push("cpm magnetoelastic")
            yield from self._me_gen()
            _range_pop()
        _range_push("cpm demag")
        yield from self._demag_gen()
        _range_pop()
        _range_push("cpm gauss-seidel projection")
        yield from self._gs_gen(Hext)
        _range_pop()
        self.nstep += 1

    # ------------------------------------------------------------------ results
    def solve_infos(self):
        raw = self.info.cpu().numpy()
        return [decode_info(raw[k]) for k in range(len(SOLVE_NAMES))]

    def iterations(self):
        """CG iterations of the last step in the reference's solve order."""
        inf = self.solve_infos()
        its = []
        if self.ME:
            its.append(inf[0]["iters"][0])
        its.append(inf[1]["iters"][0])
        its += inf[2]["iters"][:3]
        its.append(inf[3]["iters"][0])
        its.append(inf[4]["iters"][0])
        its += inf[5]["iters"][:3]
        return its

    def solve_slots(self):
        """(k, A, b, x) of every solve a step requests, in order (slot k = SOLVE_NAMES[k])."""
        pairs = [(0, self.A_el, self.b_el, self.u), (1, self.A_demag, self.bdemag, self.U),
                 (2, self.A1, self.b3, self.g), (3, self.A1, self.b1, self.g1s), (4, self.A1, self.b1, self.g2s),
                 (5, self.A2, self.b3, self.mss)]
        return [t for t in pairs if self.ME or t[0] != 0]

    def check(self):
        """Synchronise and raise the reference's RuntimeError if a solve failed."""
        return self.check_infos(self.solve_infos())

    def check_infos(self, inf):
        """Raise the reference's RuntimeError for the first failed solve in decoded infos."""
        for k, A, b, x in self.solve_slots():
            nrhs = 3 if k in (2, 5) else 1
            raise_for(inf[k], A, b, x, system=SOLVE_NAMES[k], nrhs=nrhs)
        return inf


class CGRequest:
    """One linear solve of an LLG step: A x = b with the solver's tolerances and warm-start flag."""

    __slots__ = ("run", "A", "b", "x", "k")

    def __init__(self, run, A, b, x, k):
        self.run, self.A, self.b, self.x, self.k = run, A, b, x, k

    @property
    def kind(self):
        return (getattr(self.A, "ncomp", 0), 1 if self.b.dim() == 1 else self.b.shape[1], self.k)

    def execute(self):
        self.run._cg(self.A, self.b, self.x, self.k)


def effective_field(solver: LLGSolver, m, Hext, dt=None):
    """Module-level form of the field evaluation: returns (f, f dt + m) for m (n,3)."""
    m = torch.as_tensor(m, dtype=torch.float64, device=solver.dev).contiguous()
    f = torch.empty_like(m)
    t = torch.empty_like(m)
    solver.effective_field(m, solver.p.dt if dt is None else dt, Hext, f_out=f, t_out=t)
    return f, t


def magnetoelastic_strain(solver: LLGSolver):
    return solver.magnetoelastic_strain()


def demag_field(solver: LLGSolver):
    return solver.demag_field()


def gs_projection_step(solver: LLGSolver, Hext):
    return solver.gs_projection_step(Hext)
