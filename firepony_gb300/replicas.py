"""Replica mode across GPUs: the path does not shard, so each GPU of a node runs an independent job (its own
engine, batches and tables) and no data crosses GPUs. A job set's time is the slowest rank's; its throughput
is the reads of all ranks over that time. The only collective is this max of timings."""
from __future__ import annotations


def job_throughput(ms_value: float, t_e2e: float, reads_per_rank: int, world: int, device: str = "cuda"):
    """Returns (reads/s with inputs resident, end-to-end reads/s, max device ms, max end-to-end s) over all ranks.
    With world > 1 the default process group must be initialised (NCCL with device "cuda", gloo with "cpu")."""
    if world > 1:
        import torch
        import torch.distributed as dist
        x = torch.tensor([float(ms_value), float(t_e2e)], dtype=torch.float64, device=device)
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        ms_value, t_e2e = float(x[0]), float(x[1])
    total = reads_per_rank * world
    return total / (ms_value / 1e3), total / t_e2e, ms_value, t_e2e
