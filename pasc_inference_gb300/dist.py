"""Multi-process helpers for runs launched one rank per GPU (torchrun / torch.distributed.run).

The FEM-H1 SPG path does not shard in this library: N GPUs run N independent replicas of the
workload ("replicas only").  Ranks exchange nothing on the data path; these helpers only
synchronise the timed region (barrier) and combine timings (max over ranks) on the host with
the gloo backend, so no GPU collective is ever issued."""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass
class RankInfo:
    rank: int = 0
    world_size: int = 1
    local_rank: int = 0
    initialised: bool = False


def rank_info() -> RankInfo:
    return RankInfo(rank=int(os.environ.get("RANK", "0")),
                    world_size=int(os.environ.get("WORLD_SIZE", "1")),
                    local_rank=int(os.environ.get("LOCAL_RANK", "0")))


def init(timeout_s: float = 600.0) -> RankInfo:
    """Joins the process group when launched with WORLD_SIZE > 1 (gloo over 127.0.0.1)."""
    info = rank_info()
    if info.world_size > 1:
        import datetime

        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        os.environ.setdefault("MASTER_PORT", "29531")
        if not dist.is_initialized():
            dist.init_process_group("gloo", rank=info.rank, world_size=info.world_size,
                                    timeout=datetime.timedelta(seconds=timeout_s))
        info.initialised = True
    return info


def barrier(info: RankInfo) -> None:
    if info.world_size > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(info: RankInfo, value: float) -> float:
    if info.world_size <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(info: RankInfo, value: float) -> float:
    if info.world_size <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def finalize(info: RankInfo) -> None:
    if info.world_size > 1:
        import torch.distributed as dist
        if dist.is_initialized():
            dist.destroy_process_group()
