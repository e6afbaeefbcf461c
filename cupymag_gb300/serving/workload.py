"""Synthetic serving workload: seeded hex LLG runs arriving as a Poisson process.

Each request is an independent LLG run: a periodic hex grid of edge n drawn
log-uniformly from [16, 96], a centred cubic non-magnetic defect of seeded
size 0..n/4, magnetoelastic coupling (with the [111] rotation) on for a
seeded half of the requests, a seeded initial magnetisation and a linear
field sweep +B0 -> -B0 along x over a fixed number of steps with a seeded
amplitude B0 in [0.05, 0.2] T.  Material and solver parameters are those of
the 128^3 magnetoelastic workload.  Gaps between arrivals are exponential
with the given rate.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from ..workloads import hex_params, seeded_m0, sweep_field


@dataclass(frozen=True)
class Request:
    rid: int
    edge: int
    defect: int
    ME: bool
    B0: float
    steps: int
    seed: int
    arrival: float = 0.0   # seconds after the start of serving

    def params(self):
        return hex_params(self.edge, self.defect, self.ME, self.ME)

    def fields(self, p=None):
        p = p or self.params()
        return np.array([sweep_field(p, s, self.steps, self.B0) for s in range(self.steps)], dtype=np.float64)

    def initial_m(self, n_dof, defect_dofs):
        """The run's initial magnetisation (n_dof, 3): normalise((1,0,0) + N(0, 1e-3)) from the request's
        seed, zero on the defect DOFs."""
        return seeded_m0(n_dof, defect_dofs, self.seed)

    @property
    def n_dof(self):
        return self.edge ** 3


def serving_requests(count=256, rate=20.0, seed=2024, edge_range=(16, 96), steps=100, B0_range=(0.05, 0.2),
                     me_fraction=0.5):
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=count)
    arrival = np.cumsum(gaps) - gaps[0]
    lo, hi = edge_range
    edges = np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), size=count))).astype(int)
    defects = [int(rng.integers(0, e // 4 + 1)) for e in edges]
    me = np.zeros(count, dtype=bool)
    me[rng.permutation(count)[:int(round(count * me_fraction))]] = True
    B0 = rng.uniform(*B0_range, size=count)
    seeds = rng.integers(0, 2 ** 31 - 1, size=count)
    return [Request(i, int(edges[i]), defects[i], bool(me[i]), float(B0[i]), int(steps), int(seeds[i]),
                    float(arrival[i])) for i in range(count)]
