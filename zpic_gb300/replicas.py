"""Independent replicas of a run, one process per GPU.

The em2d step is not sharded. Under torchrun every rank runs its own copy of
the workload, with no communication on the data path. Ranks only meet at
barriers around a timed region, and to take the slowest rank's time. The
throughput of the whole job is then the sum of the ranks' work divided by
that time (weak scaling).
"""
from __future__ import annotations

import os


class Replicas:
    def __init__(self, backend=None):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        self.device = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as dist

            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
                self.device = f"cuda:{self.local}"
            dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def allmax(self, v: float) -> float:
        """the largest value over the ranks"""
        if not self.dist:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, units_per_rank: float, seconds: float) -> float:
        """whole-job units per second: every rank's units over the slowest
        rank's time"""
        return units_per_rank * self.world / self.allmax(seconds)

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()
            self.dist = None
