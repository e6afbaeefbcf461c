"""World-size-2 gloo runs of the multi-GPU host logic: replica timing and request sharding."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, fn, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, fn(rank, world)))
    finally:
        dist.destroy_process_group()


def _run(fn, world=2):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, fn, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return out


def _replicas(rank, world):
    import bench
    # rank r "took" 1 + r seconds for 10 steps: the job's rate uses the slowest rank
    return bench.max_over_ranks(1.0 + rank), bench.replica_throughput(10, 1.0 + rank)


def test_replica_timing_takes_the_slowest_rank():
    out = _run(_replicas)
    for r in (0, 1):
        assert out[r][0] == 2.0
        assert out[r][1] == pytest.approx(2 * 10 / 2.0)


def _shards(rank, world):
    from cupymag_gb300.serving.engine import ServeStats
    from cupymag_gb300.serving.router import combine_stats, shard_requests
    from cupymag_gb300.serving.workload import serving_requests
    reqs = serving_requests(count=40)
    mine = shard_requests(reqs, world, rank)
    st = ServeStats(steps=sum(r.steps for r in mine), requests=len(mine), makespan_s=10.0 + rank)
    agg = combine_stats(st, [r.arrival + 1.0 for r in mine])
    return sorted(r.rid for r in mine), agg


def test_request_sharding_covers_every_request_once():
    out = _run(_shards)
    a, b = out[0][0], out[1][0]
    assert not set(a) & set(b)
    assert sorted(a + b) == list(range(40))
    assert len(a) > 5 and len(b) > 5
    for r in (0, 1):
        agg = out[r][1]
        assert agg["requests"] == 40 and agg["steps"] == 4000 and agg["ranks"] == 2
        assert agg["makespan_s"] == 11.0
        assert agg["steps_per_s"] == pytest.approx(4000 / 11.0)
    assert out[0][1]["latency_p99_s"] == out[1][1]["latency_p99_s"]


def test_sharding_balances_estimated_work():
    from cupymag_gb300.serving.router import request_work, shard_requests
    from cupymag_gb300.serving.workload import serving_requests
    reqs = serving_requests()
    loads = [sum(request_work(r) for r in shard_requests(reqs, 4, k)) for k in range(4)]
    assert max(loads) / min(loads) < 1.5
    assert sum(len(shard_requests(reqs, 4, k)) for k in range(4)) == len(reqs)
