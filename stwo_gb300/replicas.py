"""Multi-GPU as independent replicas (one process per GPU, launched by torchrun).

Proving shards by whole proofs: every stage of one proof runs on one device, so N GPUs run N
independent replicas and exchange nothing on the data path. The only collectives are the
timing ones: a barrier around the timed region and the maximum step time over ranks, from which
the whole-job rate is the work of all ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass
class Ranks:
    world: int
    rank: int
    local: int

    @staticmethod
    def from_env() -> "Ranks":
        return Ranks(int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
                     int(os.environ.get("LOCAL_RANK", "0")))


def barrier(ranks: Ranks, cuda: bool = True) -> None:
    import torch

    if ranks.world > 1:
        torch.distributed.barrier()
    if cuda:
        torch.cuda.synchronize()


def max_over_ranks(v: float, ranks: Ranks, device: str = "cuda") -> float:
    """The largest of the ranks' values (all ranks receive it)."""
    if ranks.world == 1:
        return v
    import torch

    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, ranks: Ranks, slowest_step_s: float) -> float:
    """Weak scaling: every rank does the same work; the job rate counts all of it."""
    return units_per_rank * ranks.world / slowest_step_s
