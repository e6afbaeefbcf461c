"""Benchmark: LLG steps/s of the GSPM step on one GB300 (replicas across GPUs).

Default workload: 128^3 hex with magnetoelastic coupling and the [111]
rotation (cfg "hex128_me"), in the precision form on the matrix-free stencil
operators: the elastic and demag solves by FFT inside FP64 refinement, the
Gauss-Seidel solves by FP32 CG with FP64 reliable updates.  A "step" is one
Gauss-Seidel-projection LLG step at the next field of the 500-step sweep,
with all operators and state resident in HBM.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
                  [--precision DP|IR] [--operators csr|stencil] [--impl ours|reference]

value:  steps/s over K steps timed with CUDA events (device-resident inputs;
        about 1.5 GB resident at 128^3 with every operator matrix-free, far
        above the L2, so no flush is needed); max over ranks.
e2e:    the same K steps again, from a copy of the state they started from,
        through the public API with the magnetisation copied in from pinned
        host memory and the new m and <m> read back every step (wall clock);
        bitwise_same_m_as_timed_steps records that they reproduce the timed m.
fp64:   the same steps from the same m0 in plain FP64 on the same GPU, with
        max |m - m_FP64| and the relative <m> error.
roofline: the CG launches (dominant kernel): algorithmic bytes per launch
        (stencil CG: 44 B per unknown-iteration in FP32, 88 B in FP64; FFT
        solve: fft_launch_bytes) / the CUDA-event launch time, against
        MEASURED_PEAKS.json.
serving: a sample of the 256-request serving stream through the engine,
        beside the same requests run one at a time in plain FP64.
cpu_baseline: the CPU oracle (NumPy/SciPy restatement of the reference's step)
        on this machine's host cores.
--impl reference: the oracle's CPU step as the whole measurement, every CG
        uncapped (the reference itself needs CuPy and a CUDA GPU; its CPU path is
        the oracle); at 128^3 one cold then one timed step, about 4 min each.
Multi-GPU: independent replicas (one per rank, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LLG steps/s & SpMV HBM GB/s vs plain FP64 at |m| err<=1e-6; serving p50/p99"

def elastic_launch_traffic(n_dof, elastic, steps):
    """DRAM bytes per elasticity-solve launch (ncu bytes per unknown-iteration x this run's iterations)
    and a description with the algorithmic bytes of the same launch; elastic = [bytes, ms, iterations]
    summed over `steps` steps."""
    its = elastic[2] / steps
    traffic = float(round(IR_STENCIL_DRAM_BYTES_PER_UNKNOWN_ITER * 3 * n_dof * its))
    detail = {"unit": "bytes per elasticity launch", "launch_iterations": round(its, 1),
              "algorithmic_bytes_per_launch": float(round(elastic[0] / steps)),
              "source": f"ncu dram__bytes_read.sum + dram__bytes_write.sum per unknown-iteration "
                        f"({IR_STENCIL_DRAM_BYTES_PER_UNKNOWN_ITER} B, one capture of a 300-iteration elastic "
                        f"128^3 launch) x 3 n unknowns x this run's iterations"}
    return traffic, detail


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.proc is None:
            return False
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        for line in out.splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)
        return False

    def summary(self):
        rows = getattr(self, "rows", [])
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1])]
        mx = [num(r[2]) for r in rows if num(r[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def max_over_ranks(x: float) -> float:
    """The maximum of x over the process group (x itself without one); NCCL on GPUs, gloo on the host."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def replica_throughput(steps_per_rank: int, seconds: float) -> float:
    """Whole-job steps/s of independent replicas: all ranks' steps over the slowest rank's time."""
    import torch.distributed as dist
    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    return world * steps_per_rank / max_over_ranks(seconds)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def spmv_bytes(A, nvec):
    ip = A.indptr.element_size()
    return A.nnz * (8 + 4) + (A.shape[0] + 1) * ip + nvec * (A.shape[1] * 8 + A.shape[0] * 8)


def stencil_launch_bytes(A, nvec, iters, outer, fp32, df=0):
    """Algorithmic bytes of a matrix-free CG launch: vector passes only (flags and coefficients are cached).

    FP64 CG: 88 B per unknown and iteration (q = A p: read p, write q; x, r update: read 4, write 2;
    p update: read 2, write 1).  FP32 inner iterations: 44 B; each refinement sweep: 48 B (residual: read
    x, b, write r, p, d in FP32; x += d), and 8 B more for each of the df sweeps on a double-float residual
    (the fold also writes x split into two floats, which that residual reads in place of x).
    """
    u = A.shape[0] * nvec
    if fp32:
        return u * (44 * iters + 48 * max(outer, 1) + 8 * df)
    return u * (88 * iters + 24)


# DRAM bytes (read + write) per unknown and iteration of the FP32 stencil CG, measured with ncu on a GB300
# (dram__bytes_read.sum + dram__bytes_write.sum of a 300-iteration elastic 128^3 launch / (300 x unknowns):
# (10.91 + 28.00) GB / 300 / 6.29 M for the current kernel); the vectors fit the L2 about half way, so this
# is below the 44 algorithmic bytes.  Traffic of a launch is this figure times its unknowns and iterations
# (it grows in proportion at a fixed grid size).
IR_STENCIL_DRAM_BYTES_PER_UNKNOWN_ITER = 20.6


def fft_launch_bytes(A, iters, outer, warm=True, carry=False):
    """Algorithmic bytes of an FFT solve launch (csrc/fftcg.cu), per unknown.

    Direct refinement (operators pinned at one anchor node, the default): each FP64 residual 20 B (read
    x, b; write r) plus 8 B with a residual carry (write t), one more residual than steps; the first of a
    cold start reads no x (x = 0: 12 B, and 8 B more with a carry, which also takes b); the first of a
    warm start with a carry is read from it (b, the carry's b and t; write r, b, t: 44 B) and, when it
    already meets the test, confirmed by an FP64 residual.  Each step 52 B plus the inverse symbol of the
    half spectrum (4 B elastic, 2 B scalar): slab pass 1 (read r 4, write the half spectrum 4), pass 2
    (read and write it, 8), pass 3 (read it 4, write z 4, read r 4), x += z + shift (read z 4, x 16); read
    b once (8).  Preconditioned CG: inner iteration 120 B + the full symbol (8 B elastic, 4 B scalar),
    each FP64 residual and fold 44 B (36 B for a cold start's first)."""
    u = A.shape[0]
    if getattr(A, "anchor", -1) >= 0:
        steps = max(outer, 0)
        ct = 8 if carry else 0
        if warm and carry:
            first, rest = 44, max(steps, 1)
        else:
            first, rest = (20 if warm else 12) + 2 * ct, steps
        return u * (first + (20 + ct) * rest + (52 + (4 if A.ncomp == 3 else 2)) * steps + 8)
    per_inner = 120 + (8 if A.ncomp == 3 else 4)
    return u * (per_inner * iters + 44 * max(outer, 1) - (0 if warm else 8) + 8)


def cg_launch_bytes(A, nvec, iters, warm):
    n = A.shape[0]
    per_it = spmv_bytes(A, nvec) + 6 * n * 8 * nvec
    head = (spmv_bytes(A, nvec) + 3 * n * 8 * nvec) if warm else 2 * n * 8 * nvec
    return head + iters * per_it


def workload_config(args, w, S, p, world, ops_kind):
    """The `config` object both arms print: the workload and its sizes (no run-specific values)."""
    return {"workload": args.workload,
            "mesh": (f"hex {w['n']}^3 periodic, defect {w['defect']}^3" if S.structured else
                     f"{w['n']}^3 cube of Kuhn tets ({S.n_elements} tets, interior nodes jittered "
                     f"+-{w['jitter']} h), {w['defect']} defect, seeded rotation"),
            "n_dof": S.n_dof, "magnetoelastic": w["ME"], "rot111": w["rot111"],
            "precision": args.precision, "operators": ops_kind, "tol": p.tol,
            "sweep": f"+{w['B0']} T -> -{w['B0']} T over {w['steps']} steps",
            "l2": ("inputs larger than L2 (the step's vectors alone are far above its 126 MB)"
                   if S.n_dof * 33 * 8 > 4 * 126e6 else
                   "inputs smaller than L2, not flushed (a latency-bound side workload, not the headline)"),
            "parallelism": f"replicas x{world}"}


def threaded_oracle_cg(axpy):
    """oracle.cg.solve_cg with the CG's element-wise updates as row blocks on every host thread (the
    products are threaded by the operators themselves); the same arithmetic as the single-threaded
    oracle, so the same iterates."""
    from oracle.cg import cg

    def solve(A, b, M=None, x0=None, tol=1e-7, maxiter=5000, use_init=False, system=None, record=None, dot=None):
        x, info = cg(A, b, x0=(x0 if use_init else None), tol=tol, maxiter=maxiter, record=record, axpy=axpy,
                     dot=dot)
        if info != 0:
            raise RuntimeError(f"Error! CG for {system} did not converge. info={info}.")
        return x
    return solve


# ------------------------------------------------------------------ CPU oracle sample
def cpu_sample(p, S, iters_per_solve, cap=3):
    """Time one oracle step at full size with every CG capped at `cap` iterations; the sparse products
    and the CG's element-wise updates run as row blocks on every host core (bit-identical to the
    single-threaded step; the dot products stay single-threaded NumPy)."""
    import numpy as np
    import oracle.cg as OC
    import oracle.llg as OL
    from oracle.threaded import ThreadedAxpy, threaded_operators
    from oracle.volume_average import VolumeAverage as OVA
    from cupymag_gb300.workloads import seeded_m0

    ops, pool, threads = threaded_operators(S.host_operators())
    axpy = ThreadedAxpy(pool, threads)
    Avg = OVA(S.node_coords_np, S.elements_np, S.global_id_np)
    m0 = seeded_m0(S.n_dof, S.DefDOF, seed=1234)
    st = OL.LLGState(m0, Avg.average)
    times = []
    orig = OL.solve_cg

    def capped(A, b, **kw):
        t0 = time.perf_counter()
        x, _ = OC.cg(A, b, x0=kw.get("x0") if kw.get("use_init") else None, tol=0.0, maxiter=cap, axpy=axpy)
        times.append(time.perf_counter() - t0)
        return x

    OL.solve_cg = capped
    try:
        t0 = time.perf_counter()
        OL.llg_step(st, ops, Avg.average, p, p.Hext, S.DefDOF)
        t_step = time.perf_counter() - t0
    finally:
        OL.solve_cg = orig
        pool.shutdown()
    t_fixed = t_step - sum(times)
    per_it = [t / (cap + 1) for t in times]  # one SpMV for r0 plus `cap` iterations
    est = t_fixed + sum((it + 1) * pi for it, pi in zip(iters_per_solve, per_it))
    try:
        import threadpoolctl  # noqa: F401
        from threadpoolctl import threadpool_info
        blas = max([d.get("num_threads", 1) for d in threadpool_info()] or [1])
    except Exception:
        blas = None
    return {"steps_per_s": 1.0 / est, "t_step_est_s": est, "t_fixed_s": t_fixed, "t_sample_s": t_step,
            "per_iter_s": per_it, "cores": threads, "blas_threads": blas}


# ------------------------------------------------------------------ plain FP64 beside the precision form
def fp64_check(args, S, p, L, m0, fields):
    """The same steps from the same m0 with every solve in FP64 (stencil operators on structured grids,
    the same CSR matrices otherwise); returns (solver, ms)."""
    import torch
    from cupymag_gb300.physics.llg import LLGSolver
    ops = (L.A_demag, L.Fx, L.Fy, L.Fz, L.Deriv, L.A1, L.A2, L.F1, L.A_el, L.F_el, L.Avg)
    R = LLGSolver(S, p, precision="DP", operators="stencil" if S.structured else "csr", ops=ops)
    R.set_magnetization(torch.as_tensor(m0))
    for s in range(args.warmup):
        R.step(fields[s])
        R.check()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for s in range(args.warmup, args.warmup + args.steps):
        R.step(fields[s])
    e1.record(stream)
    torch.cuda.synchronize()
    R.check()
    return R, e0.elapsed_time(e1)


# ------------------------------------------------------------------ serving sample
def serving_sample(args):
    """The first K requests of the serving stream through the engine (FP32 + FP64 refinement, real-time
    Poisson arrivals), beside the same requests run one at a time in plain FP64 (each for its first few
    steps, extrapolated to the full sweep with its own setup time)."""
    import numpy as np
    from cupymag_gb300.serving import ServingEngine, run_sequential, serving_requests
    import torch.distributed as dist
    from cupymag_gb300.serving.router import combine_stats, shard_requests
    world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
    rank = dist.get_rank() if world > 1 else 0
    reqs = shard_requests(serving_requests()[:args.serve_requests], world, rank)
    res, st = ServingEngine("IR", hbm_budget_gb=args.hbm_budget_gb).serve(reqs, realtime=True)
    agg = combine_stats(st, [r.latency for r in res.values() if r.error is None]) if world > 1 else None
    seq, _ = run_sequential(reqs, precision="DP", max_steps=args.seq_steps)
    t_seq, steps, errs = 0.0, 0, []
    for r in reqs:
        q = seq[r.rid]
        t_steps = q.completed - q.admitted - q.setup_s
        t_seq += q.setup_s + t_steps * r.steps / max(q.steps, 1)
        steps += r.steps
        a, b = res[r.rid].hist[:q.steps, :3], q.hist[:, :3]
        if len(a) == len(b) and len(b):
            errs.append(float(np.abs(a - b).max() / np.abs(b).max()))
    seq_sps = steps / t_seq if t_seq > 0 else None
    if world > 1:
        # sequential baseline of the whole job: every rank's requests one after another on its own GPU
        seq_sps = sum_over_ranks(steps) / max_over_ranks(t_seq) if t_seq > 0 else None
        st.makespan_s, st.steps = agg["makespan_s"], agg["steps"]
        st.latency_p50_s, st.latency_p99_s, st.failed = agg["latency_p50_s"], agg["latency_p99_s"], agg["failed"]
    edges = [r.edge for r in reqs]
    return {"requests": len(reqs) if world == 1 else agg["requests"], "ranks": world,
            "sharding": "whole requests, greedy least-loaded by estimated work, no data-path collective",
            "arrivals": "Poisson 20/s", "edges": f"{min(edges)}..{max(edges)}",
            "magnetoelastic": sum(r.ME for r in reqs), "steps_per_request": reqs[0].steps,
            "precision": "f32+f64", "makespan_s": round(st.makespan_s, 3), "steps_per_s": round(st.steps_per_s, 2),
            "latency_p50_s": round(st.latency_p50_s, 3), "latency_p99_s": round(st.latency_p99_s, 3),
            "failed": st.failed, "mean_batch": round(st.mean_batch, 2), "max_batch": st.max_batch,
            "graph_steps": st.graph_steps, "eager_steps": st.eager_steps, "captures": st.captures,
            "graph_error": st.graph_error, "blockdiag_launches": st.blockdiag_launches,
            "peak_budget_gb": round(st.peak_budget_gb, 2), "hbm_budget_gb": args.hbm_budget_gb,
            "sequential_fp64_steps_per_s": None if seq_sps is None else round(seq_sps, 3),
            "speedup_vs_sequential": None if not seq_sps else round(st.steps_per_s / seq_sps, 2),
            "sequential_sample": (f"each request alone in plain FP64 (stencil operators, host check per step) for "
                                  f"its first {args.seq_steps} steps, time per step x {reqs[0].steps} + setup"),
            "avg_m_rel_err_vs_fp64_first_steps": max(errs) if errs else None}


# ------------------------------------------------------------------ our arm
def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from cupymag_gb300.build import build
    build()
    from cupymag_gb300 import _native as N
    N.load()
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    from cupymag_gb300.physics.llg import LLGSolver
    from cupymag_gb300.workloads import seeded_m0, sweep_field, workload

    p, w = workload(args.workload)
    t_setup = time.perf_counter()
    S = SimulationOperators(p, mesh=w.get("mesh"))
    ops_kind = args.operators or ("csr" if args.precision == "DP" or not S.structured else "stencil")
    L = LLGSolver(S, p, precision=args.precision, operators=ops_kind)
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t_setup
    m0 = seeded_m0(S.n_dof, S.DefDOF, seed=1234 + rank)
    L.set_magnetization(torch.as_tensor(m0))
    nsw = w["steps"]
    fields = [sweep_field(p, s % nsw, nsw, w["B0"]) for s in range(args.warmup + 2 * args.steps)]
    for s in range(args.warmup):
        L.step(fields[s])
        L.check()
    resident_bytes = torch.cuda.memory_allocated()   # operators, state and CG workspaces
    stream = torch.cuda.current_stream()
    # per-CG-launch events and solver infos for the roofline of the CG kernel
    cg_events = []
    orig_cg = L._cg

    def timed_cg(A, b, x, k):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        orig_cg(A, b, x, k)
        e1.record(stream)
        cg_events.append((A, 3 if b.dim() == 2 else 1, k, e0, e1))

    # the run's state before the timed steps: the end-to-end leg below repeats the same steps from it
    snapshot = {k: t.clone() for k, t in L._state_tensors().items()}
    nstep0 = L.nstep
    L._cg = timed_cg
    info_hist = []
    warm_hist = []
    launches0 = L.launches
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        t0.record(stream)
        for s in range(args.warmup, args.warmup + args.steps):
            warm_hist.append(L.use_init.clone())
            L.step(fields[s])
            info_hist.append(L.info.clone())
        t1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    L._cg = orig_cg
    launches = L.launches - launches0
    L.check()
    m_timed, avg_timed = L.m.clone(), L.avg_m.clone()
    ms = t0.elapsed_time(t1)
    # max over ranks
    ms_max = 1e3 * max_over_ranks(ms / 1e3)
    value = replica_throughput(args.steps, ms / 1e3)

    # roofline of the CG kernel
    from cupymag_gb300.solvers.linear_solvers import decode_info
    per_step = len(cg_events) // args.steps
    from cupymag_gb300.physics.llg import FFT_SLOTS
    tot_bytes, tot_ms, dom, kern = 0.0, 0.0, {}, {}
    for i, (A, nv, k, e0, e1) in enumerate(cg_events):
        s = i // per_step
        inf = decode_info(info_hist[s][k].cpu().numpy())
        warm = bool(warm_hist[s].item())
        its = max(inf["iters"][:nv])
        fp32 = args.precision != "DP"
        if hasattr(A, "ncomp") and fp32 and L.precond == "fft" and k in FFT_SLOTS and nv == 1 and \
                A.fft_plan() is not None:
            kn, b = "cg_stencil_fft_kernel", fft_launch_bytes(A, its, inf["outer"], warm, k in L.carry)
        elif hasattr(A, "ncomp"):
            kn = "cg_stencil_ir_kernel" if fp32 else "cg_stencil_fp64_kernel"
            b = stencil_launch_bytes(A, nv, its, inf["outer"], fp32, inf["df_updates"])
        else:
            kn, b = ("cg_ir_kernel" if fp32 else "cg_fp64_kernel"), cg_launch_bytes(A, nv, its, warm)
        d = e0.elapsed_time(e1)
        tot_bytes += b
        tot_ms += d
        key = ["elasticity", "demag", "A1x3", "A1", "A1", "A2x3"][k]
        dd = dom.setdefault(key, [0.0, 0.0, 0, kn])
        dd[0] += b
        dd[1] += d
        dd[2] += its
        kk = kern.setdefault(kn, [0.0, 0.0, 0])
        kk[0] += b
        kk[1] += d
        kk[2] += 1
    its_step, upd_step, dfu_step = [], [], []
    for s in range(args.steps):
        infs = [decode_info(info_hist[s][k].cpu().numpy()) for k in range(6)]
        row = ([infs[0]["iters"][0]] if L.ME else []) + [infs[1]["iters"][0]] + infs[2]["iters"][:3] + \
              [infs[3]["iters"][0], infs[4]["iters"][0]] + infs[5]["iters"][:3]
        its_step.append(row)
        upd_step.append([infs[k]["outer"] for k in range(6)])
        dfu_step.append([infs[k]["df_updates"] for k in range(6)])
    its_mean = [float(np.mean([r[j] for r in its_step])) for j in range(len(its_step[0]))]
    peak, peak_kind = peaks()
    # the dominant kernel: the CG kernel with the most time in the timed steps
    kname = max(kern, key=lambda kn: kern[kn][1])
    kb, kms, kl = kern[kname]
    achieved = kb / (kms / 1e3) / 1e9
    traffic, traffic_detail = None, None
    if kname == "cg_stencil_ir_kernel" and "elasticity" in dom and dom["elasticity"][3] == kname and \
            args.workload == "hex128_me":
        # DRAM bytes per elasticity launch, scaled from the ncu capture of the same kernel on this grid
        traffic, traffic_detail = elastic_launch_traffic(S.n_dof, dom["elasticity"], args.steps)
    roof = {"kernel": kname, "bound": "hbm",
            "achieved": round(achieved, 1), "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic, "traffic_detail": traffic_detail,
            "launches_per_step": round(kl / args.steps, 1),
            "share_of_step": round(kms / ms, 4), "cg_share_of_step": round(tot_ms / ms, 4),
            "kernels": {kn: {"GB/s": round(v[0] / (v[1] / 1e3) / 1e9, 1), "ms_per_step": round(v[1] / args.steps, 3),
                             "frac": round(v[0] / (v[1] / 1e3) / 1e9 / peak, 4)} for kn, v in kern.items()},
            "per_solve": {k: {"kernel": v[3], "GB/s": round(v[0] / (v[1] / 1e3) / 1e9, 1),
                              "ms": round(v[1] / args.steps, 3), "iters": round(v[2] / args.steps, 1)}
                          for k, v in dom.items()}}

    # e2e: public API with host buffers, the timed steps again from the state they started from
    for k, t in L._state_tensors().items():
        t.copy_(snapshot[k])
    L.nstep = nstep0
    host_m = torch.empty((S.n_dof, 3), dtype=torch.float64).pin_memory()
    host_m.copy_(L.m.cpu())
    host_avg = torch.empty(3, dtype=torch.float64).pin_memory()
    torch.cuda.synchronize()
    tw = time.perf_counter()
    for s in range(args.warmup, args.warmup + args.steps):
        L.m.copy_(host_m, non_blocking=True)
        L.step(fields[s])
        host_m.copy_(L.m, non_blocking=True)
        host_avg.copy_(L.avg_m, non_blocking=True)
        torch.cuda.current_stream().synchronize()
    e2e_s = time.perf_counter() - tw
    L.check()
    e2e_value = replica_throughput(args.steps, e2e_s)
    e2e_same = bool(torch.equal(L.m, m_timed))

    fp64 = None
    # plain FP64 CG iterations per solve of one step (the reference's unpreconditioned CG): the
    # extrapolation of the CPU oracle sample
    fp64_iters = its_mean if args.precision == "DP" else None
    if args.precision != "DP" and not args.no_fp64_check:
        R, ms64 = fp64_check(args, S, p, L, m0, fields)
        v64 = args.steps / (ms64 / 1e3)
        err_m = float((m_timed - R.m).abs().max())
        err_avg = float((avg_timed - R.avg_m).abs().max() / R.avg_m.abs().max())
        fp64_iters = R.iterations()
        fp64 = {"steps_per_s": round(v64, 4), "ms_per_step": round(ms64 / args.steps, 3), "operators": R.operators,
                "speedup": round(value / world / v64, 3), "max_abs_m_err": err_m, "avg_m_rel_err": err_avg,
                "after_steps": args.warmup + args.steps, "bound": 1e-6}
        del R
        torch.cuda.empty_cache()

    resident_gb = resident_bytes / 1e9
    op_gb = sum(x.nbytes() for x in [L.A_demag, L.A1, L.A2, L.F1, L.Fx, L.F_el] + ([L.A_el] if L.ME else [])
                if x is not None and hasattr(x, "nbytes")) / 1e9
    serving = None
    if args.serve_requests > 0 and S.structured:
        # every rank serves its share of the request stream (no data-path collective)
        del L
        torch.cuda.empty_cache()
        serving = serving_sample(args)
    line = None
    if rank == 0:
        cpu = None
        if world == 1 and not args.no_cpu_baseline and fp64_iters is None:
            cpu = {"value": None, "unit": "steps/s", "cores": 1, "kind": "port",
                   "sample": "not taken: no plain FP64 iteration counts (run without --no-fp64-check)"}
        elif world == 1 and not args.no_cpu_baseline:
            try:
                cs = cpu_sample(p, S, fp64_iters)
                cpu = {"value": round(cs["steps_per_s"], 6), "unit": "steps/s", "cores": cs["cores"],
                       "kind": "port",
                       "sample": (f"oracle step at {w['n']}^3 with every CG capped at 3 iterations "
                                  f"({cs['t_sample_s']:.1f} s), per-solve iteration time x the plain FP64 CG "
                                  f"iterations of this run's last FP64 step {[round(x, 1) for x in fp64_iters]} "
                                  f"(the reference's unpreconditioned CG); sparse products and CG updates as "
                                  f"row blocks on {cs['cores']} host threads (SciPy and NumPy release the GIL), dot "
                                  f"products single-threaded, BLAS threads {cs['blas_threads']}"),
                       "t_step_est_s": round(cs["t_step_est_s"], 2)}
            except Exception as e:  # the baseline is reported, never required
                cpu = {"value": None, "unit": "steps/s", "cores": 1, "kind": "port", "sample": f"failed: {e}"}
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "DP" else "f32+f64",
            "data": "synthetic (seeded m0 = normalise((1,0,0)+N(0,1e-3)), fixed field sweep)",
            "config": workload_config(args, w, S, p, world, ops_kind),
            "run": {"timed_steps": f"{args.warmup}..{args.warmup + args.steps - 1}",
                    "resident_gb": round(resident_gb, 2), "csr_operator_gb": round(op_gb, 2),
                    "setup_s": round(t_setup, 1), "cg_iterations_per_step": [round(x, 1) for x in its_mean],
                    "warm_started_steps": int(sum(int(w.item()) for w in warm_hist)),
                    # per solve slot (elasticity, demag, g1n/g2n/g3n, g1star, g2star, A2 x3): reliable
                    # updates (FFT solves: refinement steps), and the updates taken on a double-float residual
                    "updates_per_step": [round(float(np.mean([r[k] for r in upd_step])), 1) for k in range(6)],
                    "df_updates_per_step": [round(float(np.mean([r[k] for r in dfu_step])), 1) for k in range(6)]},
            "e2e": {"value": round(e2e_value, 4), "unit": "steps/s", "steps": f"{args.warmup}..{args.warmup + args.steps - 1}",
                    "bitwise_same_m_as_timed_steps": e2e_same,
                    "h2d_bytes_per_step": S.n_dof * 3 * 8, "d2h_bytes_per_step": S.n_dof * 3 * 8 + 24},
            "gpu_launches": launches,
            "fp64": fp64,
            "serving": serving,
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return line


# ------------------------------------------------------------------ reference arm
def run_reference(args):
    """The reference's CPU path for the step, measured: the oracle (the reference's step restated in
    NumPy/SciPy; the reference itself needs CuPy and a CUDA GPU) with operators assembled on the host,
    sparse products and CG updates on every host thread, every CG uncapped.  One cold step, then the
    timed warm-started steps.  Workloads of a million DOFs or more time one step after one cold step
    (a full 128^3 step takes minutes on the host cores), whatever --steps and --warmup ask."""
    rank, world, local = dist_env()
    if rank != 0:
        return None
    import numpy as np
    import oracle.llg as OL
    from oracle.threaded import ThreadedAxpy, threaded_operators
    from oracle.volume_average import VolumeAverage as OVA
    from cupymag_gb300.core.assemble_simulation_operators import SimulationOperators
    from cupymag_gb300.workloads import seeded_m0, sweep_field, workload

    p, w = workload(args.workload)
    t0 = time.perf_counter()
    S = SimulationOperators(p, device="cpu", mesh=w.get("mesh"))
    # row blocks on every host thread pay off for large grids only (thread hand-offs cost more than
    # a 32^3 product)
    ops, pool, threads = threaded_operators(S.host_operators(), None if S.n_dof >= 200_000 else 1)
    Avg = OVA(S.node_coords_np, S.elements_np, S.global_id_np)
    t_setup = time.perf_counter() - t0
    big = S.n_dof >= 1_000_000
    warmup, steps = (1, 1) if big else (args.warmup, args.steps)
    nsw = w["steps"]
    st = OL.LLGState(seeded_m0(S.n_dof, S.DefDOF, seed=1234), Avg.average)
    orig = OL.solve_cg
    OL.solve_cg = threaded_oracle_cg(ThreadedAxpy(pool, threads))
    times, iters = [], []
    try:
        for s in range(warmup + steps):
            st.iters = []
            ts = time.perf_counter()
            OL.llg_step(st, ops, Avg.average, p, sweep_field(p, s % nsw, nsw, w["B0"]), S.DefDOF)
            if s >= warmup:
                times.append(time.perf_counter() - ts)
                iters.append(list(st.iters))
    finally:
        OL.solve_cg = orig
        pool.shutdown()
    t = float(np.mean(times))
    value = 1.0 / t
    ops_kind = args.operators or ("csr" if args.precision == "DP" or not S.structured else "stencil")
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": "steps/s", "n_gpus": world,
            "steps": steps, "warmup": warmup, "ms_per_step": round(t * 1e3, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, w, S, p, world, ops_kind),
            "run": {"steps_note": (f"{warmup} cold step then {steps} timed warm-started step(s)"
                                   + (f" (--steps {args.steps} --warmup {args.warmup} cut: a full {w['n']}^3 "
                                      f"oracle step takes minutes on the host cores)" if big else "")),
                    "setup_s": round(t_setup, 1), "cg_iterations_per_step": iters,
                    "measured": "every CG uncapped, wall time of the whole step; nothing extrapolated"},
            "cpu_baseline": {"value": round(value, 6), "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": (f"CPU oracle (NumPy/SciPy restatement of the reference step, whose own "
                                        f"arithmetic is CuPy on a GPU): {steps} full warm-started {w['n']}^3 "
                                        f"step(s) after {warmup} cold one, operators assembled on the host, "
                                        f"sparse products and CG updates as row blocks on {threads} host threads, "
                                        f"dot products single-threaded NumPy")},
            "e2e": {"value": round(value, 6), "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="hex128_me")
    ap.add_argument("--precision", default="IR", choices=["DP", "IR"],
                    help="IR: FP32 CG with FP64 reliable updates (default); DP: plain FP64")
    ap.add_argument("--operators", default=None, choices=["csr", "stencil"],
                    help="solved operators as CSR or matrix-free stencils (default: csr for DP, stencil for IR)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true", help="skip the plain FP64 run beside the IR form")
    ap.add_argument("--serve-requests", type=int, default=32,
                    help="requests of the serving stream to serve after the step benchmark (0: none)")
    ap.add_argument("--seq-steps", type=int, default=5, help="steps per request of the sequential FP64 sample")
    ap.add_argument("--hbm-budget-gb", type=float, default=150.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
