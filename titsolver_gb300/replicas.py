"""Multi-GPU runs of the WCSPH path are independent replicas: the path has no
data exchange between GPUs (every tank is advanced on one device), so N
ranks each run their own copy and only host-side bookkeeping is shared: a
barrier around the timed region, the maximum time and the summed work.

One process per GPU, launched by torch.distributed.run; the rank reads
RANK / LOCAL_RANK / WORLD_SIZE / MASTER_* from the environment.  With one
rank nothing here touches torch.distributed.
"""

from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass
class Ranks:
    rank: int = 0
    local_rank: int = 0
    world_size: int = 1
    dist: object | None = None

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def _reduce(self, value: float, op_name: str) -> float:
        if self.dist is None:
            return float(value)
        import torch

        t = torch.tensor([float(value)], dtype=torch.float64)
        self.dist.all_reduce(t, op=getattr(self.dist.ReduceOp, op_name))
        return float(t.item())

    def max(self, value: float) -> float:
        return self._reduce(value, "MAX")

    def sum(self, value: float) -> float:
        return self._reduce(value, "SUM")

    def close(self) -> None:
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def init_from_env(backend: str = "gloo") -> Ranks:
    """Join the process group when WORLD_SIZE > 1.  Host-only collectives
    (barrier, max, sum of scalars) go over gloo by default."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return Ranks()
    import torch.distributed as dist

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend, world_size=world,
                            rank=int(os.environ["RANK"]))
    return Ranks(rank=int(os.environ["RANK"]),
                 local_rank=int(os.environ.get("LOCAL_RANK", os.environ["RANK"])),
                 world_size=world, dist=dist)


def aggregate(units_per_rank: float, seconds_per_rank: float, ranks: Ranks) -> tuple[float, float]:
    """Whole-job throughput: units of all ranks over the slowest rank's time."""
    total_units = ranks.sum(units_per_rank)
    t_max = ranks.max(seconds_per_rank)
    return total_units / t_max if t_max > 0 else 0.0, t_max
