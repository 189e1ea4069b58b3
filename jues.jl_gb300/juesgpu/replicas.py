"""Replica runs: one process per GPU, each rank an independent problem.

The hot path has no data-parallel split of one system (a sweep at nbf=200 fits one GB300), so a
multi-GPU run is N replicas: each rank solves its own seeded system, or its own share of a batch
of independent systems, and only timings cross ranks (a barrier before and after the timed
region and a max over ranks).  torch.distributed is the transport: NCCL under torchrun on GPUs,
gloo for the host-side tests.
"""
import os
from dataclasses import dataclass
from typing import Any, Optional, Sequence


@dataclass
class Replicas:
    world_size: int = 1
    rank: int = 0
    local_rank: int = 0
    backend: Optional[str] = None
    dist: Any = None          # torch.distributed when world_size > 1

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def max(self, x: float) -> float:
        """Largest x over the ranks (every rank gets it)."""
        if self.dist is None:
            return float(x)
        import torch
        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def shard(self, items: Sequence) -> list:
        """This rank's share of independent units: every rank-th item from this rank's index,
        so the shares partition the sequence and differ in size by at most one."""
        return list(items[self.rank::self.world_size])

    def close(self) -> None:
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def setup(backend: Optional[str] = None) -> Replicas:
    """Read WORLD_SIZE / RANK / LOCAL_RANK (torchrun's variables) and join the process group
    when there is more than one rank (backend: nccl by default, gloo for CPU runs)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws <= 1:
        return Replicas(1, 0, local)
    import torch.distributed as dist
    backend = backend or "nccl"
    if backend == "nccl":
        import torch
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return Replicas(ws, rank, local, backend, dist)
