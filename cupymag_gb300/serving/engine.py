"""Continuous-batching serving loop for LLG runs on one GPU.

Requests (independent LLG runs: a hex mesh, a field sweep, a seeded initial
magnetisation) arrive over time.  The engine admits a waiting request as soon
as a slot is free and its estimated device memory fits the HBM budget, keeps
every admitted run's state (m, u, fields, warm-start flag, CG vectors)
resident on the device, and advances all admitted runs together, one
Gauss-Seidel-projection step (cupymag/core/Micromagnetics.py:110-307) at a
time:

* each run's element-wise kernels run on its own data; each of the step's
  solve slots (elasticity, demag, A1 x3, g1*, g2*, A2 x3) is one block-diagonal
  CG launch over all runs that have that solve, per coefficient table and size
  class (runs within a factor ``size_ratio`` of each other in DOFs share a
  launch, since a launch lasts as long as its slowest system);
* runs are grouped by size class; a group's step is captured in a CUDA graph
  once per group composition (the first step after a change runs eagerly,
  the following ones replay the graph); the applied field follows each run's
  sweep through a device step counter; the loop steps the group that has
  used the least GPU time so far, so small runs are not held to the pace of
  large ones;
* after each step one device-to-host copy returns every run's solver status;
  a run that finished its sweep is retired (slot and memory released, its
  final m and <m> history copied out) and waiting requests are admitted.

A run's result does not depend on which other runs share its batch: the
block-diagonal solver reduces each system in a fixed order of its own, and
every other kernel of a run reads and writes only that run's data.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from .. import _native as N
from ..core.assemble_simulation_operators import SimulationOperators
from ..physics.llg import FFT_SLOTS, INNER_TOL, SOLVE_NAMES, LLGSolver
from ..solvers.linear_solvers import decode_info
from .blockdiag import BlockDiagPlan, BlockSystem, coef_key, work_bytes

NSLOTS = len(SOLVE_NAMES)
# Runs of at least this many DOFs solve elasticity and demag with the FFT solver, one launch per run;
# smaller runs keep them in the block-diagonal launches (latency-bound either way).
FFT_MIN_DOFS = 32 ** 3


def estimate_bytes(p, precision="IR") -> int:
    """Device bytes one run holds.  Every operator of a served run is matrix-free (stencils of the
    solved operators, F1, Fx, Fy, Fz and F_el), so per DOF it is: 33 FP64 vectors of the step (51 with
    magnetoelastic coupling), the volume-average weights, five flag arrays and the defect mask, the
    block-diagonal CG vectors of the largest solve (3n unknowns: five FP32 or three FP64 vectors), in the
    precision form the residual carries of the demag and elastic solves (b and t of each), and for runs
    that solve elasticity and demag with the FFT solver its workspace and plans."""
    n = int(p.Nx) * int(p.Ny) * int(p.Nz)
    per = (51 if p.ME else 33) * 8 + 8 + 6
    per += 3 * (20 if precision != "DP" else 24)
    if precision != "DP":
        per += 2 * 8 * (4 if p.ME else 1)
    if precision != "DP" and n >= FFT_MIN_DOFS:
        # FFT solves: workspace (five FP32 vectors and a complex field of 3n unknowns) and the plans'
        # inverse symbols (6 floats per DOF elastic, 1 demag)
        per += 3 * (20 + 8) + 4 * (6 + 1)
    return int(per * n * 1.05) + (8 << 20)


@dataclass
class Run:
    req: object
    solver: LLGSolver
    slot: int
    work: torch.Tensor
    est_bytes: int
    t_admit: float
    steps_done: int = 0
    error: str = None


@dataclass
class Result:
    rid: int
    arrival: float
    admitted: float
    completed: float
    steps: int
    hist: np.ndarray            # (steps, 4): <m> and sumsq after each step
    m: np.ndarray = None        # final magnetisation (n, 3)
    error: str = None
    setup_s: float = 0.0

    @property
    def latency(self):
        return self.completed - self.arrival


@dataclass
class ServeStats:
    makespan_s: float = 0.0
    steps: int = 0
    requests: int = 0
    failed: int = 0
    latency_p50_s: float = 0.0
    latency_p99_s: float = 0.0
    graph_steps: int = 0
    eager_steps: int = 0
    captures: int = 0
    batch_steps: int = 0
    mean_batch: float = 0.0
    max_batch: int = 0
    peak_budget_gb: float = 0.0
    graph_error: str = None
    blockdiag_launches: int = 0
    fft_launches: int = 0
    extra: dict = field(default_factory=dict)

    @property
    def steps_per_s(self):
        return self.steps / self.makespan_s if self.makespan_s > 0 else 0.0


class OperatorCache:
    """The matrix-free operators of a run, shared by runs of the same grid, defect and material.

    Admission builds a run's mesh, DOF map, defect DOFs and stencil operators
    (cupymag/core/assemble_simulation_operators.py:42-107) once per key
    (edge, defect size and centre, coupling, rotation, the solved operators'
    material and time-step constants) and hands every later run with that key
    the same read-only objects.  Least recently used keys leave when the cache
    holds `capacity` of them."""

    def __init__(self, device, capacity=64):
        self.dev = device
        self.capacity = int(capacity)
        self._d = {}
        self.hits = self.misses = 0

    @staticmethod
    def key(p):
        return (int(p.Nx), int(p.Ny), int(p.Nz), int(p.Ndx), int(p.Ndy), int(p.Ndz),
                None if p.defect_center is None else tuple(float(v) for v in p.defect_center), bool(p.ME),
                bool(p.rot111), float(p.alpha1), float(p.alpha2), float(p.c11), float(p.c12), float(p.c44))

    def get(self, p):
        k = self.key(p)
        hit = self._d.pop(k, None)
        if hit is None:
            self.misses += 1
            S = SimulationOperators(p, device=self.dev)
            hit = (S, S.stencil_step_operators())
            if len(self._d) >= self.capacity:
                self._d.pop(next(iter(self._d)))
        else:
            self.hits += 1
        self._d[k] = hit
        return hit


class _Group:
    """Runs of one size class: stepped together, with their own plans and CUDA graph."""

    def __init__(self, cls):
        self.cls = cls
        self.runs = []
        self.plans = None
        self.graph = None
        self.eager_since_change = 0
        self.gpu_s = 0.0          # measured step time spent on this group (scheduling key)

    def changed(self):
        self.plans = None
        self.graph = None
        self.eager_since_change = 0


class ServingEngine:
    def __init__(self, precision="IR", hbm_budget_gb=150.0, max_runs=64, use_graphs=True, device=None,
                 keep_m=False, size_ratio=4.0, time_launches=False):
        N.require_cuda()
        self.dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.precision = "DP" if precision == "DP" else "IR"
        self.budget = float(hbm_budget_gb) * 1e9
        self.max_runs = int(max_runs)
        self.use_graphs = bool(use_graphs)
        self.keep_m = keep_m
        # runs whose DOF counts lie in the same power of size_ratio form one group (None: a
        # single group); a launch lasts as long as its slowest system, and groups are stepped
        # independently, the one with the least step time spent so far first
        self.size_ratio = size_ratio
        # diagnostic: CUDA events around every block-diagonal launch (steps run eagerly);
        # per (slot, group) milliseconds accumulate in stats.extra["launch_ms"]
        self.time_launches = bool(time_launches)
        if self.time_launches:
            self.use_graphs = False
        self._events = []
        self.infos = torch.zeros((self.max_runs, NSLOTS, N.CG_INFO_BYTES), dtype=torch.uint8, device=self.dev)
        self.free = list(range(self.max_runs))[::-1]
        self.groups = {}
        self.used = 0
        self.stats = ServeStats()
        self.cache = OperatorCache(self.dev)

    @property
    def active(self):
        return [r for g in self.groups.values() for r in g.runs]

    def _cls(self, n):
        return 0 if not self.size_ratio else int(math.floor(math.log(n) / math.log(self.size_ratio)))

    # ------------------------------------------------------------------ admission
    def fits(self, req) -> bool:
        return bool(self.free) and self.used + estimate_bytes(req.params(), self.precision) <= self.budget

    def admit(self, req, now):
        p = req.params()
        est = estimate_bytes(p, self.precision)
        S, ops = self.cache.get(p)
        slot = self.free.pop()
        self.infos[slot].zero_()
        L = LLGSolver(S, p, precision=self.precision, operators="stencil", ops=ops, info=self.infos[slot])
        L.set_field_schedule(req.fields(p))
        L.set_magnetization(torch.as_tensor(req.initial_m(S.n_dof, S.DefDOF)))
        work = torch.empty(work_bytes((p.Nx, p.Ny, p.Nz), 3, 1, self.precision), dtype=torch.uint8,
                           device=self.dev)
        run = Run(req, L, slot, work, est, now)
        cls = self._cls(L.n)
        g = self.groups.get(cls)
        if g is None:
            g = self.groups[cls] = _Group(cls)
            # a new group starts level with the least-served group, so it does not monopolise the GPU
            busy = [h.gpu_s for h in self.groups.values() if h.runs and h is not g]
            g.gpu_s = min(busy) if busy else 0.0
        g.runs.append(run)
        g.changed()
        self.used += est
        self.stats.peak_budget_gb = max(self.stats.peak_budget_gb, self.used / 1e9)
        return run

    # ------------------------------------------------------------------ one batched step of a group
    def _fft_solve(self, L, k, A):
        """Whether slot k of run L is solved alone with the FFT solver (precision form,
        elasticity or demag, a grid of at least FFT_MIN_DOFS DOFs with an FFT plan) instead of in the
        block-diagonal launch.  It depends on the run alone, so a run's result is the same in any mix."""
        return (self.precision == "IR" and L.precond == "fft" and k in FFT_SLOTS and L.n >= FFT_MIN_DOFS
                and A.fft_plan() is not None)

    def _build_plans(self, g):
        sys_by_key = {}
        fft = {k: [] for k in range(NSLOTS)}
        for run in g.runs:
            L = run.solver
            for k, A, b, x in L.solve_slots():
                if self._fft_solve(L, k, A):
                    fft[k].append((run, A, b, x))
                    continue
                key = (k, A.ncomp, 1 if b.dim() == 1 else int(b.shape[1]), coef_key(A))
                sys_by_key.setdefault(key, []).append(
                    BlockSystem(A, b, x, L.info[k], run.work, L.p.tol, L.p.maxiter, L.use_init))
        plans = {k: [] for k in range(NSLOTS)}
        for key, systems in sys_by_key.items():
            plans[key[0]].append(BlockDiagPlan(systems, self.precision, device=self.dev, inner_tol=INNER_TOL[key[0]]))
        g.plans = plans
        g.fft = fft

    def _step_runs(self, g):
        """Launch one step of every run of the group: element-wise kernels per run, one CG launch per slot."""
        gens = [r.solver.step_gen(None) for r in g.runs]
        cur = [next(x, None) for x in gens]
        for k in range(NSLOTS):
            idx = [i for i, q in enumerate(cur) if q is not None and q.k == k]
            if not idx:
                continue
            for plan in g.plans[k]:
                if self.time_launches:
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    plan.launch()
                    e1.record()
                    self._events.append((f"slot{k}/group{g.cls}", e0, e1))
                else:
                    plan.launch()
                self.stats.blockdiag_launches += 1
            for run, A, b, x in g.fft[k]:
                run.solver._cg(A, b, x, k)
                self.stats.fft_launches += 1
            for i in idx:
                cur[i] = next(gens[i], None)
        if any(q is not None for q in cur):
            raise RuntimeError("a run requested a solve outside the step's slot order")

    def step(self, g=None):
        """Advance every run of group g (all groups when None) by one step (asynchronous)."""
        if g is None:
            for h in list(self.groups.values()):
                if h.runs:
                    self.step(h)
            return
        if g.plans is None:
            self._build_plans(g)
        if g.graph is None and self.use_graphs and g.eager_since_change >= 1:
            try:
                gr = torch.cuda.CUDAGraph()
                with torch.cuda.graph(gr):
                    self._step_runs(g)
                g.graph = gr
                self.stats.captures += 1
            except Exception as e:  # capture unsupported: keep stepping eagerly
                self.use_graphs = False
                self.stats.graph_error = f"{type(e).__name__}: {e}"
                torch.cuda.synchronize(self.dev)
        if g.graph is not None:
            g.graph.replay()
            self.stats.graph_steps += 1
        else:
            self._step_runs(g)
            self.stats.eager_steps += 1
            g.eager_since_change += 1
        b = len(g.runs)
        self.stats.batch_steps += 1
        self.stats.mean_batch += b
        self.stats.max_batch = max(self.stats.max_batch, len(self.active))
        for r in g.runs:
            r.steps_done += 1

    # ------------------------------------------------------------------ completion
    def _poll(self, now, results, groups=None):
        """Read every run's solver status (one copy) and retire finished or failed runs."""
        raw = self.infos.cpu().numpy()
        if self._events:
            lm = self.stats.extra.setdefault("launch_ms", {})
            for name, e0, e1 in self._events:
                lm[name] = lm.get(name, 0.0) + e0.elapsed_time(e1)
            self._events = []
        for g in (groups if groups is not None else list(self.groups.values())):
            retired = False
            for run in list(g.runs):
                err = None
                for k, *_ in run.solver.solve_slots():
                    d = decode_info(raw[run.slot, k])
                    if d["status"] != N.CPM_OK:
                        err = (f"step {run.steps_done}: CG for {SOLVE_NAMES[k]} ended with "
                               f"{N.STATUS_NAMES.get(d['status'], d['status'])} (iterations {d['iters']})")
                        break
                if err is None and run.steps_done < run.req.steps:
                    continue
                L = run.solver
                results[run.req.rid] = Result(run.req.rid, run.req.arrival, run.t_admit, now, run.steps_done,
                                              L.hist[:run.steps_done].cpu().numpy(),
                                              L.m.cpu().numpy() if self.keep_m else None, err)
                g.runs.remove(run)
                self.free.append(run.slot)
                self.used -= run.est_bytes
                retired = True
            if retired:
                g.changed()

    def serve(self, requests, realtime=True):
        """Serve the requests (arrival offsets in seconds when realtime); returns ({rid: Result}, ServeStats)."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        results = {}
        for r in list(pending):
            if estimate_bytes(r.params(), self.precision) > self.budget:
                pending.remove(r)
                results[r.rid] = Result(r.rid, r.arrival, 0.0, 0.0, 0, np.zeros((0, 4)),
                                        error="request exceeds the HBM budget")
        torch.cuda.synchronize(self.dev)
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0  # noqa: E731

        def admit_arrived():
            while pending and (not realtime or pending[0].arrival <= clock()) and self.fits(pending[0]):
                self.admit(pending.popleft(), clock())

        while pending or any(g.runs for g in self.groups.values()):
            admit_arrived()
            live = [g for g in self.groups.values() if g.runs]
            if not live:
                if pending:
                    time.sleep(max(0.0, min(pending[0].arrival - clock(), 0.05)))
                continue
            g = min(live, key=lambda h: (h.gpu_s, h.cls))
            ts = time.perf_counter()
            self.step(g)
            # requests that arrived meanwhile are set up while the step runs on the GPU (all of
            # them at once: spreading admissions over turns churns group compositions, and every
            # change costs a plan build, an eager step and a graph capture)
            admit_arrived()
            torch.cuda.synchronize(self.dev)
            dt = time.perf_counter() - ts
            g.gpu_s += dt
            # per size class: seconds, batched steps and run-steps (where the makespan goes)
            gs = self.stats.extra.setdefault("groups", {}).setdefault(str(g.cls), [0.0, 0, 0])
            gs[0] += dt
            gs[1] += 1
            gs[2] += len(g.runs)
            self._poll(clock(), results, [g])
        st = self.stats
        done = [r for r in results.values() if r.completed > 0]
        first = min((r.arrival for r in done), default=0.0)
        st.makespan_s = max((r.completed for r in done), default=0.0) - first
        st.steps = sum(r.steps for r in done if r.error is None)
        st.requests = len(results)
        st.failed = sum(1 for r in results.values() if r.error)
        lat = np.array([r.latency for r in done if r.error is None])
        if lat.size:
            st.latency_p50_s = float(np.percentile(lat, 50))
            st.latency_p99_s = float(np.percentile(lat, 99))
        if st.batch_steps:
            st.mean_batch /= st.batch_steps
        return results, st


def run_sequential(requests, precision="DP", operators="stencil", device=None, keep_m=False, max_steps=None):
    """Each request alone, one after another, with a host check after every step (the unbatched baseline).

    Returns ({rid: Result}, total seconds); times include each run's setup
    (Result.setup_s).  max_steps stops every run early (a timing sample)."""
    N.require_cuda()
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    results = {}
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for req in requests:
        ts = time.perf_counter() - t0
        p = req.params()
        S = SimulationOperators(p, device=dev)
        L = LLGSolver(S, p, precision=precision, operators=operators)
        L.set_field_schedule(req.fields(p))
        L.set_magnetization(torch.as_tensor(req.initial_m(S.n_dof, S.DefDOF)))
        torch.cuda.synchronize(dev)
        t_setup = time.perf_counter() - t0 - ts
        err = None
        for _ in range(req.steps if max_steps is None else min(req.steps, max_steps)):
            L.step(None)
            try:
                L.check()
            except RuntimeError as e:
                err = str(e)
                break
        torch.cuda.synchronize(dev)
        te = time.perf_counter() - t0
        done = int(L.hstep.item())
        results[req.rid] = Result(req.rid, ts, ts, te, done, L.hist[:done].cpu().numpy(),
                                  L.m.cpu().numpy() if keep_m else None, err, t_setup)
    return results, time.perf_counter() - t0
