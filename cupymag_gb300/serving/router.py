"""Request-level sharding of the serving loop across GPUs (one engine per rank).

LLG runs are independent, so serving shards by request: every rank computes
the same deterministic assignment of whole requests to ranks and serves its
share with its own ``ServingEngine``; nothing on the data path crosses GPUs.
Only the summary statistics are combined (a sum of completed steps and
requests, the maximum makespan and the latencies gathered for percentiles),
with ``torch.distributed`` collectives on whatever backend the process group
uses (NCCL on GPUs, gloo on the host).
"""
from __future__ import annotations

import numpy as np


def request_work(req) -> float:
    """Relative cost of a request: steps x DOFs x (elastic solve weight when coupled)."""
    n = req.edge ** 3
    return req.steps * n * (4.0 if req.ME else 1.0) * req.edge ** 0.5


def shard_requests(requests, world: int, rank: int):
    """The requests rank `rank` of `world` serves: greedy least-loaded assignment in arrival order.

    Deterministic (ties go to the lowest rank), so every rank computes the
    same partition without communication; each request lands on exactly one
    rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    load = np.zeros(world)
    mine = []
    for req in sorted(requests, key=lambda r: (r.arrival, r.rid)):
        k = int(np.argmin(load))
        load[k] += request_work(req)
        if k == rank:
            mine.append(req)
    return mine


def combine_stats(stats, latencies, group=None):
    """Aggregate one rank's ServeStats and latency list over the process group.

    Returns a dict with the whole-job steps, requests, failures, makespan
    (maximum over ranks), steps/s (total steps / that makespan) and the p50/p99
    of all ranks' latencies."""
    import torch
    import torch.distributed as dist

    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else "cpu"
    sums = torch.tensor([float(stats.steps), float(stats.requests), float(stats.failed)], dtype=torch.float64,
                        device=dev)
    mx = torch.tensor([float(stats.makespan_s)], dtype=torch.float64, device=dev)
    dist.all_reduce(sums, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(mx, op=dist.ReduceOp.MAX, group=group)
    world = dist.get_world_size(group)
    gathered = [None] * world
    dist.all_gather_object(gathered, [float(x) for x in latencies], group=group)
    lat = np.array([x for part in gathered for x in part])
    makespan = float(mx.item())
    steps = float(sums[0].item())
    return {"steps": int(steps), "requests": int(sums[1].item()), "failed": int(sums[2].item()),
            "makespan_s": makespan, "steps_per_s": steps / makespan if makespan > 0 else 0.0,
            "latency_p50_s": float(np.percentile(lat, 50)) if lat.size else 0.0,
            "latency_p99_s": float(np.percentile(lat, 99)) if lat.size else 0.0, "ranks": world}
