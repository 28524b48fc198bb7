"""Host logic of the N-GPU bench on CPU: the material sharding, and the two-rank aggregation
(sum of work, max of time) over a world-size-2 gloo group. The path has no data-path
collective; each rank optimises its own materials."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _bench():
    sys.path.insert(0, ROOT)
    import bench

    return bench


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_shard_covers_every_material_once_and_balances(world):
    bench = _bench()
    specs = bench.workload_specs(64)
    costs = [bench.material_cost(r, v) for r, v in specs]
    parts = bench.shard(costs, world)
    assert len(parts) == world
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(64))
    loads = [sum(costs[i] for i in p) for p in parts]
    # greedy largest-first: no rank exceeds the mean by more than the largest material
    assert max(loads) <= sum(costs) / world + max(costs)
    assert parts == bench.shard(costs, world)  # deterministic


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench = _bench()
        specs = bench.workload_specs(64)
        costs = [bench.material_cost(r, v) for r, v in specs]
        mine = bench.shard(costs, world)[rank]
        tv = torch.tensor([float(sum(specs[i][0] ** 2 * specs[i][1] for i in mine))], dtype=torch.float64)
        dist.all_reduce(tv)  # whole-job texel*views, as bench.py sums them
        t = torch.tensor([1.0 + rank], dtype=torch.float64)  # per-rank time
        dist.all_reduce(t, op=dist.ReduceOp.MAX)  # the job takes as long as its slowest rank
        got = [None] * world
        dist.all_gather_object(got, mine)
        if rank == 0:
            out.put((float(tv), float(t), got))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_aggregation():
    bench = _bench()
    specs = bench.workload_specs(64)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    tv, t, parts = q.get(timeout=240)
    for p in procs:
        p.join(timeout=240)
        assert p.exitcode == 0
    assert tv == float(sum(r * r * v for r, v in specs))
    assert t == 2.0
    assert sorted(i for p in parts for i in p) == list(range(64))
    assert not set(parts[0]) & set(parts[1])
