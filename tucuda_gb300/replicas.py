"""Host-side plumbing for running the filters on several GPUs.

The images (or requests) of a workload are independent, so several GPUs run
as replicas: each rank filters its own images and no data crosses between
ranks.  The only cross-rank steps are on the host: a barrier around a timed
region, the maximum of the per-rank times and the sum of the per-rank pixel
counts.  These work over whichever torch.distributed backend the caller
initialised (NCCL on GPUs, gloo on CPU ranks); with no process group they
degrade to the single-rank values.
"""


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def rank_world():
    d = _dist()
    return (d.get_rank(), d.get_world_size()) if d else (0, 1)


def shard(costs, rank, world):
    """Indices of the jobs rank `rank` of `world` runs: a deterministic
    longest-first assignment of jobs (cost = pixels, say) to the least-loaded
    rank, so every rank computes the same disjoint partition without
    communicating."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    mine = []
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        load[r] += costs[i]
        if r == rank:
            mine.append(i)
    return sorted(mine)


def _reduce(x, op_name):
    d = _dist()
    if d is None:
        return float(x)
    import torch
    dev = "cuda" if d.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    d.all_reduce(t, op=getattr(d.ReduceOp, op_name))
    return float(t.item())


def max_over_ranks(x):
    """The maximum of x over all ranks (a step time: the slowest rank)."""
    return _reduce(x, "MAX")


def sum_over_ranks(x):
    """The sum of x over all ranks (pixels processed by the whole job)."""
    return _reduce(x, "SUM")


def barrier():
    d = _dist()
    if d is not None:
        d.barrier()
