"""Multi-GPU use of the solver: one process per GPU, systems split by rank.

The systems of a batch are independent, so a batch shards by system with no
exchange at all: rank r solves systems [first, first + count) of the batch
on its own GPU with its own plan.  This replaces the reference's split of
each line over MPI ranks (one segment per rank, an all-to-all of the reduced
rows; Fortran_Original/src/mod_btdma_gpu_v2.f90:1309-1374), which a by-system
split never needs.  The systems go to ranks by the reference's own partition
rule, remainder to the low ranks (partition_1d,
CUDA_CXX_Port/src/pascal_btdma_cuda.cu:921-930; pbt_partition_1d).

In the reference GPU layout X[sys + nsys*(row + nrow*e)] the system index is
fastest, so a shard is one contiguous run of `count` values in every
(row, element) plane; `take_shard` and `put_shard` gather and scatter it.
"""
from __future__ import annotations

from . import partition_1d


def shard_of(nsys: int, world: int, rank: int) -> tuple[int, int]:
    """(first, count) of the systems rank `rank` of `world` solves."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    if nsys < world:
        return (rank, 1) if rank < nsys else (nsys, 0)
    first, last = partition_1d(0, nsys - 1, world, rank)
    return first, last - first + 1


def take_shard(x, nsys: int, first: int, count: int):
    """Systems [first, first + count) of a flat reference-layout array
    (numpy or torch), as a new contiguous array in the same layout."""
    planes = x.numel() // nsys if hasattr(x, "numel") else x.size // nsys
    v = x.reshape(planes, nsys)[:, first:first + count]
    return v.contiguous().reshape(-1) if hasattr(v, "contiguous") else v.copy().reshape(-1)


def put_shard(dst, src, nsys: int, first: int, count: int) -> None:
    """Write a shard (as returned by take_shard) back into the full array."""
    planes = dst.numel() // nsys if hasattr(dst, "numel") else dst.size // nsys
    dst.reshape(planes, nsys)[:, first:first + count] = src.reshape(planes, count)


def max_over_ranks(x: float, group=None) -> float:
    """The largest value of `x` over the ranks of the default process group
    (the slowest rank's time is the job's time); `x` itself without one."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return float(x)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
