"""Replica (data-parallel) helpers for running disjoint instance slices per GPU.

Density-matrix instances (disorder realisations, initial states, Redfield
right-hand sides) are independent, so N ranks propagate contiguous slices
of the batch with no collective on the data path.  The only exchanges are
host-side: the max-over-ranks wall time for throughput, and an optional
gather of per-instance results to rank 0.
"""
from __future__ import annotations


def shard_range(n_items: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [lo, hi) slice of ``n_items`` for ``rank`` of ``world``
    (sizes differ by at most one)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError('rank %d outside world of %d' % (rank, world))
    lo = rank * n_items // world
    hi = (rank + 1) * n_items // world
    return lo, hi


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of ``value`` over the default process group (or ``value``)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_to_rank0(tensor, device=None):
    """Concatenate per-rank slices (same trailing shape) on rank 0; other
    ranks get None.  Slices may differ in length by one."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return tensor
    world = dist.get_world_size()
    n = torch.tensor([tensor.shape[0]], dtype=torch.int64, device=device)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n)
    mx = int(max(int(s.item()) for s in sizes))
    pad = torch.zeros((mx,) + tuple(tensor.shape[1:]), dtype=tensor.dtype, device=tensor.device)
    pad[:tensor.shape[0]] = tensor
    parts = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad)
    if dist.get_rank() != 0:
        return None
    return torch.cat([p[:int(s.item())] for p, s in zip(parts, sizes)], 0)
