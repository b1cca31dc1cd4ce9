"""Multi-GPU host logic: probes are independent units, so N GPUs run N
replicas, each baking its own share of the probes; the only communication is
the final reduction of timings and counts (no data-path collective).

* ``ranks()``: (world, rank, local_rank) from the torchrun environment.
* ``shard(n, rank, world)``: probe indices of one rank (round-robin, so
  uneven probe sizes spread evenly).
* ``job_throughput(units_per_rank, seconds_per_rank)``: whole-job units/s =
  all units / the slowest rank's time (max over ranks), the weak-scaling
  figure.
* ``allreduce_max`` / ``allreduce_sum``: the reductions themselves through
  torch.distributed (NCCL on GPUs, gloo on CPU).
"""
from __future__ import annotations

import os
from typing import List, Sequence, Tuple


def ranks() -> Tuple[int, int, int]:
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(n: int, rank: int, world: int) -> List[int]:
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    return list(range(rank, n, world))


def job_throughput(units_per_rank: Sequence[float], seconds_per_rank: Sequence[float]) -> float:
    slowest = max(seconds_per_rank)
    return sum(units_per_rank) / slowest if slowest > 0 else 0.0


def _reduce(value: float, op, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def allreduce_max(value: float, device=None) -> float:
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.MAX, device)


def allreduce_sum(value: float, device=None) -> float:
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.SUM, device)
