"""Replica bookkeeping for runs on several GPUs of one node.

The path shards without any exchange: every rank holds its own copy of the
scene and traces its own samples, so the only cross-rank steps are the
timing reductions (slowest rank's time, sum of the rays) done once after the
timed region.  Rank r renders the global sample indices
[(r + k * world) * spp, ... + spp) of step k, so the ranks' samples are
disjoint and together they form one progressive accumulation (the per-sample
seeds depend only on pixel and global sample index).
"""


def sample_range(rank, world, step, spp):
    """Global sample indices [first, first + spp) that `rank` renders at `step`."""
    first = (step * world + rank) * spp
    return first, first + spp


def combine(times, counts, device=None):
    """Max over ranks of `times`, sum over ranks of `counts` (lists of floats).
    Without an initialised process group (one rank) the inputs come back."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(times), dtype=torch.float64, device=device)
    c = torch.tensor(list(counts), dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return [float(x) for x in t.cpu()], [float(x) for x in c.cpu()]
