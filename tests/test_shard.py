"""Multi-GPU form of the slice workloads, tested on CPU: the cost-balanced
slice partition (pyraft_gb300.shard) and, over a two-rank gloo process
group, that every rank derives the same disjoint, covering assignment
without communicating and that the timing reduction is the max over ranks."""
import os
import random
import socket

import pytest

from pyraft_gb300 import shard

torch = pytest.importorskip("torch")


def config5_costs(n=256, seed=3):
    rng = random.Random(seed)
    return [rng.choice([256, 512, 1024, 2048]) ** 2 * rng.randint(180, 1800) for _ in range(n)]


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_partition_covers_and_balances(world):
    costs = config5_costs()
    parts = shard.partition(costs, world)
    assert len(parts) == world
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(costs)))
    ld = shard.loads(costs, parts)
    # longest-processing-time-first: the spread is at most the largest slice
    assert max(ld) - min(ld) <= max(costs)
    assert max(ld) <= sum(costs) / world + max(costs)
    assert shard.partition(costs, world) == parts          # deterministic


def test_partition_edge_cases():
    assert shard.partition([], 3) == [[], [], []]
    assert shard.partition([5.0], 4) == [[0], [], [], []]
    assert shard.partition([1, 1, 1, 1], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        shard.partition([1.0], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        costs = config5_costs()
        mine = shard.rank_slices(costs, rank, world)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        t = shard.max_over_ranks(1.5 + rank)            # a rank's "time"
        q.put((rank, gathered, t))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_assignment_and_max():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    costs = config5_costs()
    expect = shard.partition(costs, 2)
    for rank, gathered, t in res:
        assert gathered == expect                  # every rank derived the same split
        assert t == 2.5                            # max over ranks
    assert sorted(gathered[0] + gathered[1]) == list(range(len(costs)))
