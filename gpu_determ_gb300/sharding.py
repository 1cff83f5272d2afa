"""Cells over ranks: the only multi-GPU structure this path needs.

Spatial cells are independent within a collision step, so N GPUs take
disjoint contiguous slices of the cells (weak scaling; no collective on the
data path).  Two host-side exchanges remain:

- the step time reported by a benchmark is the maximum over ranks;
- a time step shared by all ranks under the Courant rule of relax_f
  (collision_integral.cu:776-807: dt = min over every node and cell of
  courant / nu) needs the global maximum of nu: one all-reduce of one scalar
  per step, after which each rank relaxes with the fixed dt it returns.

Works with any torch.distributed backend (NCCL on GPUs, gloo on CPUs) or
without one (single process).
"""
from __future__ import annotations


def shard_cells(total: int, world: int, rank: int) -> tuple[int, int]:
    """(first cell, count) of rank's contiguous slice; the first total % world
    ranks take one extra cell."""
    if world < 1 or not 0 <= rank < world or total < 0:
        raise ValueError("need world >= 1, 0 <= rank < world, total >= 0")
    base, extra = divmod(total, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def reduce_device(dist, device=None):
    """Device of the one-scalar tensors the all-reduces use: the caller's
    choice, else the current CUDA device under NCCL (which reduces only CUDA
    tensors), else the CPU."""
    if device is not None:
        return device
    import torch
    if dist is not None and dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a host scalar over all ranks (the value itself alone)."""
    dist = _dist()
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=reduce_device(dist, device))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def global_courant_dt(local_max_nu, courant: float):
    """dt = courant / max over all ranks of the corrected collision frequency.

    local_max_nu: this rank's maximum of nu' (a float, or a one-element
    tensor on the backend's device).  Returns a Python float."""
    dist = _dist()
    import torch
    if torch.is_tensor(local_max_nu):
        t = local_max_nu.reshape(1).to(torch.float32).clone()
    else:
        t = torch.tensor([float(local_max_nu)], dtype=torch.float32, device=reduce_device(dist))
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    m = float(t.item())
    if not m > 0.0:
        raise ValueError("the collision frequency is not positive on any rank")
    return float(torch.tensor(courant, dtype=torch.float32) / torch.tensor(m, dtype=torch.float32))
