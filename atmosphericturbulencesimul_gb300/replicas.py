"""Several GPUs, one process each: the (wavelength, direction) instances are
independent given the read-only master screens, so ranks never exchange
data.  A rank either runs its own replica of the whole workload (weak
scaling, as the benchmark does) or a contiguous share of one instance list
(`partition`).  The only collective is the reduction of the timing scalars
below: the job's throughput is the frames of all ranks over the slowest
rank's time."""
from __future__ import annotations


def partition(n_items: int, rank: int, world: int) -> range:
    """Contiguous share of n_items for `rank` of `world` (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    q, r = divmod(n_items, world)
    lo = rank * q + min(rank, r)
    return range(lo, lo + q + (1 if rank < r else 0))


def aggregate(seconds: float, frames: int, group=None, device=None) -> tuple[float, int, float]:
    """(max seconds over ranks, total frames, frames/s of the job).  Without an
    initialised process group the rank's own numbers are returned."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(seconds), int(frames), float(frames) / float(seconds)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    n = torch.tensor([float(frames)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(n, op=dist.ReduceOp.SUM, group=group)
    return float(t.item()), int(round(n.item())), float(n.item()) / float(t.item())
