"""Multi-GPU evaluation is replicas only.

Instances of a mapped Function are independent (the reference's Map evaluates instance i
from ``arg[j] + i*nnz_in(j)`` with no data shared between instances, casadi/core/map.cpp:
357-381), so N GPUs each evaluate their own contiguous instance range with the tape
replicated and no exchange step; only the timing (the slowest rank) and optional result
collection cross ranks. One process per GPU (torchrun), ``torch.distributed`` for the
rank-level reductions (NCCL on GPUs, gloo on CPUs).
"""


def instance_range(n_total, rank, world):
    """Contiguous [start, stop) of the ``n_total`` instances that ``rank`` of ``world``
    evaluates (the first ``n_total % world`` ranks take one more)."""
    if world < 1 or not 0 <= rank < world or n_total < 0:
        raise ValueError("bad rank/world/instance count")
    base, extra = divmod(n_total, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard(arrays, rank, world):
    """The instance-minor arrays' (last axis) slices of this rank."""
    n = arrays[0].shape[-1]
    a, b = instance_range(n, rank, world)
    return [x[..., a:b] for x in arrays]


def max_over_ranks(value, device="cpu"):
    """The maximum of a float over all ranks of the default process group (the value itself
    without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
