"""Several GPUs: independent problem instances on independent replicas.

One grid does not shard without a halo exchange and a global sweep (the
reference gathers the whole grid to one rank for every sweep), but
independent instances do, with no collective on the data path.  `shard`
splits a list of instances across ranks by estimated cost; `aggregate` forms
the whole-job figure after the run: the work of all ranks over the slowest
rank's time (the only collective, outside the timed region).
"""
from __future__ import annotations


def shard(costs, rank: int, world: int):
    """Indices of the instances rank `rank` of `world` takes: greedy
    longest-processing-time assignment of `costs` (deterministic: ties go to
    the lower index and the lower rank)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    order = sorted(range(len(costs)), key=lambda k: (-costs[k], k))
    load = [0.0] * world
    mine = []
    for k in order:
        r = min(range(world), key=lambda q: (load[q], q))
        load[r] += costs[k]
        if r == rank:
            mine.append(k)
    return sorted(mine)


def aggregate(updates: float, seconds: float, group=None):
    """(sum of updates over ranks, max of seconds over ranks, value) with
    torch.distributed when a process group is up, else the local figures."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return updates, seconds, updates / seconds if seconds else float("nan")
    dev = torch.device("cuda", torch.cuda.current_device()) \
        if dist.get_backend(group) == "nccl" else torch.device("cpu")
    u = torch.tensor([float(updates)], dtype=torch.float64, device=dev)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    tu, tt = float(u.item()), float(t.item())
    return tu, tt, tu / tt if tt else float("nan")
