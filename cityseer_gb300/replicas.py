"""Multi-GPU form: replicas.  Sources are independent, so N ranks (one process per GPU) each run the
whole workload on their own GPU with no collective on the data path; the only exchange is the
timing reduction below (the slowest rank's time), which turns per-rank work into the whole job's
throughput.  A graph sharded by sources would add one f64 sum-reduce of the accumulator rows at
the end; with replicas there is none."""
from __future__ import annotations

import torch


def job_throughput(units_per_rank: float, seconds: float, device: torch.device | None = None) -> tuple[float, float]:
    """(units of all ranks / slowest rank's seconds, slowest seconds).  Works on one process (no
    process group) and under torch.distributed with any backend (nccl on GPUs, gloo on CPU)."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return units_per_rank / seconds, seconds
    dev = device if device is not None else torch.device("cpu")
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    u = torch.tensor([float(units_per_rank)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    t_max = float(t.item())
    return float(u.item()) / t_max, t_max
