"""Multi-GPU batch sharding, host side (CPU, gloo, world size 2): every
rank computes the same balanced partition of the instances without
communicating, and rank 0 gathers the results back in instance order."""
import os
import socket

import numpy as np
import pytest

from pdos_gb300.shard import all_gather_rows, gather_results, shard_instances


def test_partition_is_disjoint_complete_and_balanced():
    rng = np.random.default_rng(0)
    costs = list(rng.integers(200, 90000, 1000))
    for world in (1, 2, 3, 8):
        parts = [shard_instances(costs, world, r) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)
    with pytest.raises(ValueError):
        shard_instances(costs, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, costs, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard_instances(costs, world, rank)
    # stand-in for each instance's solution: computed only by its owner
    results = [{"instance": i, "obj": float(-i) * 0.5, "rank": rank} for i in mine]
    out = gather_results(results, mine, len(costs), dist)
    if rank == 0:
        q.put(out)
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_every_result_in_order():
    import torch.multiprocessing as mp
    costs = [int(c) for c in np.random.default_rng(1).integers(1, 1000, 37)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert [r["instance"] for r in out] == list(range(len(costs)))
    owners = {r["rank"] for r in out}
    assert owners == {0, 1}
    for r in out:
        assert r["instance"] in shard_instances(costs, 2, r["rank"])


def _training_rows(i, width):
    """Stand-in for instance i's solution (x, y, s) rows."""
    return np.sin(np.arange(width) * 0.37 + i) * (1.0 + i)


def _rank_rows(rank, world, port, count, width, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard_instances([1] * count, world, rank)
    local = np.stack([_training_rows(i, width) for i in mine])
    full = all_gather_rows(local, mine, count, dist)
    q.put((rank, full))
    dist.destroy_process_group()


def test_sharded_training_data_equals_unsharded():
    """The training set solved in parts by two ranks and gathered with
    all_gather_rows is, on every rank, the array one rank would make alone."""
    import torch.multiprocessing as mp
    count, width = 45, 13
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_rows, args=(r, 2, port, count, width, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    want = np.stack([_training_rows(i, width) for i in range(count)])
    assert np.array_equal(got[0], want) and np.array_equal(got[1], want)
