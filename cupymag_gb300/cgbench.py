"""Time the CG solver on one operator of a structured hex grid.

    python -m cupymag_gb300.cgbench [--edge 128] [--op A_el|A_demag|A1|A2|F_el] [--nrhs 1|3]
                                    [--precision IR|DP] [--operators stencil|csr]
                                    [--solves 3] [--maxiter 20000] [--batch 1] [--batched]
                                    [--form 0|1|2|3] [--precond fft] [--fft-layout auto|slab|passes]
                                    [--spmv] [--precond-apply] [--workload tet96_me] [--no-df]

Builds only the requested operator (the magnetoelastic 128^3 material), a
seeded right-hand side with the reference's pins (b[0] = 0 for A_demag,
b[0] = b[n] = b[2n] = 0 for A_el), and times cold-start solves with CUDA
events on the launching stream.  Prints one JSON line: iterations, reliable
updates, ms per solve, ms per iteration and the algorithmic GB/s of the
launch (vector traffic only for stencil operators, matrix + vectors for CSR).
With --batch B > 1 (or --batched) the solve is B copies of the system in one
block-diagonal launch of the serving solver.  A capped --maxiter keeps a profiled launch short; the status is then
reported, not raised.  With --operators csr --spmv it times the CSR product y = A x alone (F_el, the
magnetoelastic coupling, is available only there).
"""
from __future__ import annotations

import argparse
import json

import numpy as np
import torch


def _bytes(op, nrhs, iters, outer, fp32, csr):
    u = op.shape[0] * nrhs
    if not csr:
        return u * (44 * iters + 48 * max(outer, 1)) if fp32 else u * (88 * iters + 24)
    ip = op.indptr.element_size()
    spmv = op.nnz * ((4 if fp32 else 8) + 4) + (op.shape[0] + 1) * ip + nrhs * (op.shape[1] + op.shape[0]) * (
        4 if fp32 else 8)
    return 2 * u * 8 + iters * (spmv + 6 * u * (4 if fp32 else 8))


def _time_spmv(args, A, torch):
    """y = A x (cpm_spmv_csr) --solves times after one warm-up; algorithmic bytes: values and indices
    (12 B per non-zero), row pointers, x read and y written once."""
    nvec = 1 if args.op in ("A_el", "F_el") else args.nrhs
    cols = A.shape[1]
    x = torch.randn((cols, nvec) if nvec > 1 else (cols,), dtype=torch.float64, device="cuda")
    y = A.spmv(x)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.solves):
        A.spmv(x, out=y)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.solves
    nnz = int(A.indices.numel())
    nbytes = nnz * 12 + (A.shape[0] + 1) * A.indptr.element_size() + (A.shape[0] + cols) * 8 * nvec
    print(json.dumps({"op": args.op, "edge": args.edge, "rows": A.shape[0], "nnz": nnz, "nvec": nvec,
                      "kernel": "spmv", "ms_per_product": round(ms, 4), "GB/s": round(nbytes / ms / 1e6, 1)}))


def _time_precond(args, op, torch):
    """z = M r alone (cpm_fft_precond_apply: one launch per pass) --solves times after one warm-up."""
    from . import _native as N
    layout = {"auto": N.FFT_LAYOUT_AUTO, "slab": N.FFT_LAYOUT_SLAB, "passes": N.FFT_LAYOUT_PASSES}[args.fft_layout]
    r = torch.randn(op.shape[0], dtype=torch.float32, device="cuda")
    z = op.precondition32(r, layout=layout)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.solves):
        op.precondition32(r, z, layout=layout)
    e1.record()
    torch.cuda.synchronize()
    plan = op.fft_plan(layout)
    print(json.dumps({"op": args.op, "edge": args.edge, "n": op.shape[0], "kernel": "fft_apply",
                      "layout": {N.FFT_LAYOUT_SLAB: "slab", N.FFT_LAYOUT_PASSES: "passes"}[plan.layout],
                      "us_per_apply": round(1000 * e0.elapsed_time(e1) / args.solves, 1)}))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--edge", type=int, default=128)
    ap.add_argument("--op", default="A_el", choices=["A_el", "A_demag", "A1", "A2", "F_el"])
    ap.add_argument("--nrhs", type=int, default=1, choices=[1, 3])
    ap.add_argument("--precision", default="IR", choices=["IR", "DP"])
    ap.add_argument("--operators", default="stencil", choices=["stencil", "csr"])
    ap.add_argument("--solves", type=int, default=3)
    ap.add_argument("--maxiter", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--batched", action="store_true",
                    help="solve through the block-diagonal (serving) kernel even for --batch 1")
    ap.add_argument("--inner-tol", type=float, default=0.1,
                    help="reliable-update factor of the FP32 solver (residual drop between FP64 updates)")
    ap.add_argument("--form", type=int, default=0, choices=[0, 1, 2, 3],
                    help="FP32 stencil solver: 0 default (three barriers), 1 three-barrier, 2 two-barrier; "
                         "FFT solves: 0 direct refinement (anchored operators), 3 preconditioned CG")
    ap.add_argument("--fft-layout", default="auto", choices=["auto", "slab", "passes"],
                    help="spectrum layout of the FFT preconditioner")
    ap.add_argument("--workload", default=None,
                    help="take the grid and material of a named workload (cupymag_gb300.workloads, e.g. tet96_me "
                         "for the tet mesh; CSR operators) instead of the hex grid of --edge")
    ap.add_argument("--precond-apply", action="store_true",
                    help="time z = M r alone (the FFT apply of a stencil operator), --solves times")
    ap.add_argument("--spmv", action="store_true",
                    help="time the CSR product y = A x alone (cpm_spmv_csr), --solves times; needs --operators csr")
    ap.add_argument("--no-df", action="store_true",
                    help="FP64 residuals for every reliable update (no double-float residual passes)")
    ap.add_argument("--precond", default=None, choices=["fft"],
                    help="FP32 stencil solve preconditioned by the circulant inverse (FFT) inside FP64 refinement")
    args = ap.parse_args(argv)

    from . import _native as N
    from .core.assemble_simulation_operators import SimulationOperators
    from .solvers.linear_solvers import CGSolver, decode_info, new_info
    from .workloads import hex_params, workload
    N.require_cuda()
    N.load()
    if args.workload:
        p, w = workload(args.workload)
        S = SimulationOperators(p, mesh=w.get("mesh"))
    else:
        p = hex_params(args.edge, args.edge // 8, args.op in ("A_el", "F_el"), True)
        S = SimulationOperators(p)
    csr = args.operators == "csr"
    if args.op == "F_el" and not (csr and args.spmv):
        raise SystemExit("F_el is timed as a CSR product only (--operators csr --spmv)")
    if csr:
        op = {"A_el": lambda: S.csr_elasticity()[0], "F_el": lambda: S.csr_elasticity()[1],
              "A_demag": lambda: S.csr_demag_and_deriv()[0],
              "A1": lambda: S.csr_GS()[0], "A2": lambda: S.csr_GS()[1]}[args.op]()
    else:
        op = S.stencil_operators()[args.op]
    if args.spmv:
        if not csr:
            raise SystemExit("--spmv times the CSR product: add --operators csr")
        return _time_spmv(args, op, torch)
    if args.precond_apply:
        if csr or not hasattr(op, "precondition32"):
            raise SystemExit("--precond-apply times the FFT apply of a stencil operator")
        return _time_precond(args, op, torch)
    nrhs = 1 if args.op == "A_el" else args.nrhs
    n = op.shape[0]
    rng = np.random.default_rng(7)
    b = rng.normal(size=(n, nrhs)) if nrhs == 3 else rng.normal(size=n)
    if args.op == "A_demag":
        b[0] = 0.0
    if args.op == "A_el":
        b[[0, n // 3, 2 * n // 3]] = 0.0
    bd = torch.as_tensor(b, device="cuda").contiguous()
    stream = torch.cuda.current_stream()
    times, infos = [], []
    inner_tol = args.inner_tol
    if args.batch > 1 or args.batched:
        if csr:
            raise SystemExit("--batch needs stencil operators")
        from .serving.blockdiag import BlockDiagPlan, BlockSystem, work_bytes
        systems = []
        for _ in range(args.batch):
            systems.append(BlockSystem(op, bd, torch.zeros_like(bd), new_info(1)[0],
                                       torch.empty(work_bytes((op.nx, op.ny, op.nz), op.ncomp, nrhs,
                                                              args.precision),
                                                   dtype=torch.uint8, device="cuda"), p.tol, args.maxiter))
        plan = BlockDiagPlan(systems, args.precision, inner_tol=args.inner_tol, form=args.form)
        launch = plan.launch
        info_of = lambda: systems[0].info  # noqa: E731
    else:
        # the FFT solves' preconditioned-CG form drops its residual by 1e-4 (a circulant inverse leaves few
        # directions to resolve); plain FP32 CG restarts after the --inner-tol drop
        inner_tol = 1e-4 if args.precond else args.inner_tol
        solver = CGSolver()
        solver.df_residual = not args.no_df
        solver.inner_tol = args.inner_tol
        solver.fft_layout = {"auto": N.FFT_LAYOUT_AUTO, "slab": N.FFT_LAYOUT_SLAB,
                             "passes": N.FFT_LAYOUT_PASSES}[args.fft_layout]
        x = torch.zeros_like(bd)
        info = new_info(1)

        def launch():
            solver.launch(op, bd, x, info[0], tol=p.tol, maxiter=args.maxiter, precision=args.precision,
                          form=args.form, precond=args.precond,
                          inner_tol=inner_tol)
        info_of = lambda: info[0]  # noqa: E731
    for _ in range(args.solves):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        launch()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
        infos.append(decode_info(info_of().cpu().numpy()))
    d = infos[-1]
    its = max(d["iters"][:nrhs])
    ms = float(np.median(times))
    nb = _bytes(op, nrhs, its, d["outer"], args.precision == "IR", csr) * args.batch
    print(json.dumps({"op": args.op, "edge": args.edge, "n": n, "nrhs": nrhs, "precision": args.precision,
                      "inner_tol": inner_tol, "form": args.form, "precond": args.precond,
                      "fft_layout": args.fft_layout if args.precond else None,
                      "operators": args.operators, "batch": args.batch,
                      "kernel": "blockdiag" if args.batch > 1 or args.batched else "single",
                      "status": N.STATUS_NAMES[d["status"]],
                      "iters": its, "outer": d["outer"], "df_updates": d["df_updates"], "ms_per_solve": round(ms, 3),
                      "us_per_iter": round(1e3 * ms / max(its, 1), 2), "GB/s": round(nb / (ms / 1e3) / 1e9, 1),
                      "solve_ms": [round(t, 3) for t in times]}))


if __name__ == "__main__":
    main()
