"""The CuPyMag driver on the GB300 kernels (drop-in for cupymag/core/Micromagnetics.py:34-351).

``run(params)`` keeps the reference's control flow around the step:

* initial m (uniform or restart file), defect DOFs zeroed, <m>;
* loop while <m> . stop_direction > stop_value: one GSPM step
  (``LLGSolver.step``), then the same bookkeeping as the reference --
  output on convergence (sumsq < n * llg_accuracy_factor after more than
  llg_min_step steps, 10 with ME and 100 without) or every save_frequency
  steps, a hysteresis line ``Hext1 Hext2 Hext3 <m1> <m2> <m3>`` (A/m for H),
  and on convergence the field decrement H -= dH;
* a final hysteresis line and the last magnetisation.

Optionally ``fields`` gives a fixed per-step field schedule instead (the
benchmark sweep); ``max_steps`` bounds the loop.  VTU output is not written
(out of scope); ``write_m`` stores ``last_m`` (.h5 with h5py, else .npy).
"""
from __future__ import annotations

import os
import time

import numpy as np
import torch

from .assemble_simulation_operators import SimulationOperators
from .parameters import load_parameters


def run(params, fields=None, max_steps=None, precision=None, verbose=True, device=None):
    from ..physics.llg import LLGSolver
    from ..utils.magnetization_io import initialize_m, write_array
    from ..utils.precision_select import solver_precision

    p = params
    out_dir = p.output_dir or "."
    os.makedirs(out_dir, exist_ok=True)
    t_start = time.time()
    S = SimulationOperators(p, device=device)
    prec = precision or solver_precision(p.precision)
    L = LLGSolver(S, p, precision=prec)
    m0 = initialize_m(p.restart_m, p.restart, p.initial_magnetization, S.n_dof, S.DefDOF)
    L.set_magnetization(torch.as_tensor(m0))
    n = S.n_dof
    llg_min_step = 10 if p.ME else 100
    LLG_accuracy = n * p.LLG_accuracy_factor
    Hext = list(p.Hext)
    dH = list(p.dHext)
    stop_dir = np.asarray(p.stop_direction, dtype=np.float64)
    avg_m = L.avg_m.cpu().numpy()
    hyst = open(os.path.join(out_dir, "hysteresis.txt"), "w", buffering=1)
    hyst.write("Hext1\tHext2\tHext3\tavg_m1\tavg_m2\tavg_m3\n")
    if verbose:
        print(f"Initialized {p.grid_type} FEM mesh with #nodes={S.n_nodes}, #elements={S.n_elements}, "
              f"#defect elements={int(S.elements_np[:, -1].sum())}.")
    t_llg = time.time()
    nstep = 0
    count = 0
    total = 0
    history = []
    while avg_m @ stop_dir > p.stop_value:
        if max_steps is not None and total >= max_steps:
            break
        if fields is not None:
            if total >= len(fields):
                break
            Hext = list(fields[total])
        nstep += 1
        total += 1
        L.step(Hext)
        L.check()
        sumsq = float(L.sumsq.item())
        avg_m = L.avg_m.cpu().numpy()
        history.append(avg_m.copy())
        if verbose and nstep % 200 == 0:
            print(f"m diff L2 norm sq: {sumsq:.10f} at LLG step {nstep}")
        converged = sumsq < LLG_accuracy and nstep > llg_min_step
        if converged or nstep % p.save_frequency == 0:
            count += 1
            hyst.write(f"{Hext[0] * p.ms:.1f}\t{Hext[1] * p.ms:.1f}\t{Hext[2] * p.ms:.1f}\t"
                       f"{float(avg_m[0])!r}\t{float(avg_m[1])!r}\t{float(avg_m[2])!r}\n")
            if p.write_m:
                write_array(L.m, os.path.join(out_dir, "last_m.h5"))
            if nstep >= 5000 and verbose:
                print(f"LLG not converging at external field {Hext[0] * p.ms:.0f} A/m, at LLG step {nstep}.")
        if converged and fields is None:
            if verbose:
                print(f"LLG converge at LLG step {nstep}.")
                print(f"Current average magnetization is m1 = {avg_m[0]}, m2 = {avg_m[1]}, m3 = {avg_m[2]}.")
            Hext = [h - d for h, d in zip(Hext, dH)]
            nstep = 0
            count = 0
    hyst.write(f"{Hext[0] * p.ms:.1f}\t{Hext[1] * p.ms:.1f}\t{Hext[2] * p.ms:.1f}\t"
               f"{float(avg_m[0])!r}\t{float(avg_m[1])!r}\t{float(avg_m[2])!r}\n")
    hyst.close()
    if p.write_m:
        write_array(L.m, os.path.join(out_dir, "last_m.h5"))
    if verbose:
        now = time.time()
        print(f"Final state for average magnetization: m1 = {avg_m[0]}, m2 = {avg_m[1]}, m3 = {avg_m[2]}.")
        print(f"The code uses {now - t_start:.2f} s in total, {t_llg - t_start:.2f} s for system set up, "
              f"and {now - t_llg:.2f} for LLG calculation.")
    return {"solver": L, "avg_m": avg_m, "steps": total, "history": np.array(history)}


def main(config_path=None):
    """Entry point used by the CLI: load the YAML config and run the simulation."""
    return run(load_parameters(config_path))


if __name__ == "__main__":
    main()
