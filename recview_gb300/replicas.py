"""One process per GPU over independent slices and datasets ("replicas only").

Slices of a stack and datasets of a queue share no data, so N ranks split the units with no
data-path collective (the reference likewise gives each GPU its own worker thread and sums int32
slices on the host, source/gazoDoc.cpp:3888-3984).  The only cross-rank traffic is
bookkeeping: a barrier around the timed region and a max over ranks of the elapsed time, so
that throughput = units of all ranks / slowest rank.  These helpers are backend-agnostic (NCCL
on GPUs, gloo on CPU) so that the same code is exercised by CPU tests.
"""
from __future__ import annotations


def shard(n_units: int, world: int, rank: int) -> range:
    """Contiguous block of the n_units that rank owns; blocks differ in size by at most one."""
    if world < 1 or not 0 <= rank < world or n_units < 0:
        raise ValueError(f"bad partition: n_units={n_units} world={world} rank={rank}")
    base, extra = divmod(n_units, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def barrier() -> None:
    d = _dist()
    if d is not None and d.get_world_size() > 1:
        d.barrier()


def _reduce_device():
    import torch
    d = _dist()
    if d is not None and d.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def max_over_ranks(x: float) -> float:
    """Max of a per-rank float (elapsed time) over all ranks; x itself without a process group."""
    d = _dist()
    if d is None or d.get_world_size() == 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=_reduce_device())
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(n: int) -> int:
    """Total of a per-rank unit count over all ranks."""
    d = _dist()
    if d is None or d.get_world_size() == 1:
        return int(n)
    import torch
    t = torch.tensor([int(n)], dtype=torch.int64, device=_reduce_device())
    d.all_reduce(t, op=d.ReduceOp.SUM)
    return int(t.item())


def aggregate_rate(units_this_rank: int, seconds_this_rank: float) -> tuple[float, int, float]:
    """Whole-job throughput: (units of all ranks / slowest rank's seconds, total units, max seconds)."""
    total = sum_over_ranks(units_this_rank)
    tmax = max_over_ranks(seconds_this_rank)
    return (total / tmax if tmax > 0 else float("inf")), total, tmax
