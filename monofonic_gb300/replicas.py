"""Several GPUs of one node: replicas only.

A single IC does not shard without the global transposes of the reference's
slab decomposition (src/grid_fft.cc:115-189), and batches and serving streams
are independent realizations, so every rank runs whole realizations on its own
GPU.  Ranks meet only at a barrier and at reductions of their timings; no
collective touches the data path.  The launcher's environment (RANK,
WORLD_SIZE, LOCAL_RANK, MASTER_ADDR, MASTER_PORT) selects the rank; NCCL is the
GPU backend, gloo serves host-only use (tests).
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Any


@dataclass
class Replicas:
    world: int
    rank: int
    local: int
    backend: str | None
    dist: Any = None

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def _reduce(self, x: float, op) -> float:
        if self.dist is None:
            return float(x)
        import torch
        dev = torch.device("cuda", self.local) if self.backend == "nccl" else torch.device("cpu")
        t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max_over_ranks(self, x: float) -> float:
        """the slowest rank's value (timings: max over ranks)"""
        return self._reduce(x, None if self.dist is None else self.dist.ReduceOp.MAX)

    def sum_over_ranks(self, x: float) -> float:
        return self._reduce(x, None if self.dist is None else self.dist.ReduceOp.SUM)

    def aggregate_rate(self, units_per_rank: float, seconds: float) -> float:
        """whole-job throughput: the units all ranks processed over the
        slowest rank's time"""
        total = self.sum_over_ranks(units_per_rank)
        slowest = self.max_over_ranks(seconds)
        return total / slowest

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def init(backend: str = "nccl") -> Replicas:
    """join the job described by the launcher's environment; a single process
    (WORLD_SIZE unset or 1) needs no process group"""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    r = Replicas(world, rank, local, backend if world > 1 else None)
    if world > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group(backend)
        r.dist = dist
    return r
