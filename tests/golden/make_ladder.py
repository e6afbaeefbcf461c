"""Write the parity-ladder fixtures: oracle trajectories at the benchmark configurations' sizes.

TEST INFRASTRUCTURE.  The oracle (``oracle/``, pinned bit-for-bit to the
reference's own step by tests/test_oracle_golden.py) runs here on the CPU; the
GPU tests compare the product's FP64 step against these trajectories:

* ``ladder_hex32_plain.npz``: the 32^3 plain-FP64 workload (4^3 defect, no
  magnetoelastic coupling, seeded m0, the full 500-step +0.1 T -> -0.1 T sweep);
* ``ladder_hex32_me.npz``: 32^3 with magnetoelastic coupling and the [111]
  rotation (4^3 defect, sigma_xx = -50 MPa), the first 10 steps of that sweep.

Each file holds <m> and the CG iteration counts after every step and the final
m.  Beside the oracle's own trajectory it runs a second one whose only change is
the summation order of the CG inner products (NumPy's pairwise sum of the
element-wise products instead of BLAS ddot) and records, per step, how far that
moves m and <m>.  That is the size of a pure rounding difference at each step:
where the product's FP64 step differs from the oracle by more than 1e-10, the
tests compare the difference with this figure.

    python tests/golden/make_ladder.py            # both fixtures (about 10 minutes)
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import assembly as OA  # noqa: E402
from oracle import mesh as OM  # noqa: E402
from oracle.llg import LLGState, M_matrix, llg_step  # noqa: E402
from oracle.volume_average import VolumeAverage  # noqa: E402


def pairwise_dot(a, b):
    """a.b summed by NumPy's pairwise reduction (a different order from BLAS ddot)."""
    return float(np.add.reduce(a * b))


CASES = {
    "ladder_hex32_plain": dict(n=32, defect=4, ME=False, rot111=False, steps=500, sweep=500, B0=0.1, seed=1234),
    "ladder_hex32_me": dict(n=32, defect=4, ME=True, rot111=True, steps=10, sweep=500, B0=0.1, seed=1234),
}


def oracle_setup(p):
    coords, el = OM.hex_mesh(p.Nx, p.Ny, p.Nz, p.Ndx, p.Ndy, p.Ndz, p.defect_center)
    gid = OM.hex_periodic_map(p.Nx, p.Ny, p.Nz, coords)
    n = int(gid.max()) + 1
    defect = OM.extract_defect_dofs(el, gid)
    C = OA.voigt_C(p.c11, p.c12, p.c44, p.rot111, M_matrix()) if p.ME else None
    ops = OA.build_operators(coords, el, gid, n, defect, p.alpha1, p.alpha2, ME=p.ME, C=C)
    return n, defect, ops, VolumeAverage(coords, el, gid)


def make(name, c, out_dir):
    from cupymag_gb300.workloads import hex_params, seeded_m0, sweep_field
    p = hex_params(c["n"], c["defect"], c["ME"], c["rot111"])
    n, defect, ops, Avg = oracle_setup(p)
    m0 = seeded_m0(n, defect, seed=c["seed"])
    A = LLGState(m0, Avg.average)
    B = LLGState(m0, Avg.average)
    K = c["steps"]
    avg = np.zeros((K, 3))
    avg_b = np.zeros((K, 3))
    iters = np.full((K, 10), -1, dtype=np.int32)
    dev_m = np.zeros(K)
    dev_avg = np.zeros(K)
    t0 = time.time()
    for s in range(K):
        H = sweep_field(p, s, c["sweep"], c["B0"])
        A.iters, B.iters = [], []
        llg_step(A, ops, Avg.average, p, H, defect)
        llg_step(B, ops, Avg.average, p, H, defect, dot=pairwise_dot)
        avg[s], avg_b[s] = A.avg_m, B.avg_m
        iters[s, :len(A.iters)] = A.iters
        dev_m[s] = np.abs(A.m - B.m).max()
        dev_avg[s] = np.abs(A.avg_m - B.avg_m).max() / np.abs(A.avg_m).max()
        if s % 50 == 0 or s == K - 1:
            print(f"{name} step {s} {time.time() - t0:.0f}s its {A.iters} dev_m {dev_m[s]:.2e}", flush=True)
    path = os.path.join(out_dir, name + ".npz")
    np.savez_compressed(path, n=np.int64(c["n"]), defect=np.int64(c["defect"]), ME=np.int8(c["ME"]),
                        rot111=np.int8(c["rot111"]), steps=np.int64(K), sweep=np.int64(c["sweep"]),
                        B0=np.float64(c["B0"]), seed=np.int64(c["seed"]), avg_m=avg, iters=iters,
                        m_final=A.m, avg_m_reordered=avg_b, reorder_dev_m=dev_m, reorder_dev_avg=dev_avg)
    print("wrote", path)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", choices=sorted(CASES), action="append")
    ap.add_argument("--out", default=HERE)
    a = ap.parse_args()
    for name in a.case or sorted(CASES):
        make(name, CASES[name], a.out)


if __name__ == "__main__":
    main()
