"""Sharding a batch of independent problems over GPUs.

Instances share nothing, so a multi-GPU batch is a partition of the
instance list plus a host-side gather of the results: no collective touches
the solver's data path.  Every rank computes the same partition from the
instance costs without communicating.
"""


def shard_instances(costs, world, rank):
    """Indices (ascending) of the instances that `rank` of `world` solves.

    Greedy longest-processing-time assignment: instances in decreasing cost
    (ties by index) each go to the least-loaded rank (ties by rank number),
    which keeps every rank within one instance's cost of the mean load."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    owner = [0] * len(costs)
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += costs[i]
    return [i for i in range(len(costs)) if owner[i] == rank]


def gather_results(results, indices, count, dist):
    """Rank 0 gets every rank's results back in instance order (a list of
    `count`); other ranks get None.  `results[j]` belongs to instance
    `indices[j]`.  Host objects only, through torch.distributed's object
    gather (gloo or nccl)."""
    mine = list(zip(indices, results))
    rank = dist.get_rank()
    box = [None] * dist.get_world_size() if rank == 0 else None
    dist.gather_object(mine, box, dst=0)
    if rank != 0:
        return None
    out = [None] * count
    for part in box:
        for i, r in part:
            out[i] = r
    if any(r is None for r in out):
        raise RuntimeError("an instance was solved by no rank")
    return out


def all_gather_rows(local, indices, count, dist, device="cpu"):
    """Every rank gets every rank's rows in instance order: a (count, width)
    float64 array assembled from each rank's `local` rows (row j belongs to
    instance indices[j]).  One padded all_gather of a tensor per array and
    one of the indices -- gloo for CPU tensors, nccl for CUDA tensors.  Used
    to share the training data that the ranks solved in parts."""
    import numpy as np
    import torch
    world = dist.get_world_size()
    local = np.asarray(local, np.float64)
    width = local.shape[1]
    n_local = len(indices)
    sizes = [torch.zeros(1, dtype=torch.int64, device=device) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([n_local], dtype=torch.int64, device=device))
    cap = max(int(s.item()) for s in sizes)
    idx = torch.full((cap,), -1, dtype=torch.int64, device=device)
    idx[:n_local] = torch.as_tensor(np.asarray(indices, np.int64), device=device)
    rows = torch.zeros((cap, width), dtype=torch.float64, device=device)
    rows[:n_local] = torch.as_tensor(local, device=device)
    all_idx = [torch.empty_like(idx) for _ in range(world)]
    all_rows = [torch.empty_like(rows) for _ in range(world)]
    dist.all_gather(all_idx, idx)
    dist.all_gather(all_rows, rows)
    out = np.full((count, width), np.nan)
    seen = np.zeros(count, bool)
    for ix, rw, sz in zip(all_idx, all_rows, sizes):
        k = int(sz.item())
        ii = ix[:k].cpu().numpy()
        out[ii] = rw[:k].cpu().numpy()
        seen[ii] = True
    if not seen.all():
        raise RuntimeError("an instance's rows came from no rank")
    return out
