"""Replica bookkeeping for runs on several GPUs of one node.

The VBD step does not shard: a mesh would need a halo exchange after every colour, and the batched
form already packs many meshes onto one GPU.  A multi-GPU run is therefore N independent replicas,
one per rank (launched by torchrun: RANK, WORLD_SIZE, LOCAL_RANK and MASTER_* in the environment),
with no data exchange; the group is used only to line the ranks up before timing (barrier), to take
the slowest rank's time (max) and to add up the work of all ranks (sum).
"""

from __future__ import annotations

import os


class Replicas:
    def __init__(self, backend: str = "nccl", device=None):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.device = device
        self._dist = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group(backend)
            self._dist = dist

    @property
    def is_root(self) -> bool:
        return self.rank == 0

    def barrier(self) -> None:
        if self._dist:
            self._dist.barrier()

    def _reduce(self, value: float, op) -> float:
        if not self._dist:
            return float(value)
        import torch

        t = torch.tensor([float(value)], dtype=torch.float64, device=self.device)
        self._dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, value: float) -> float:
        """The largest value over the ranks (the time of the slowest replica)."""
        return self._reduce(value, self._dist.ReduceOp.MAX if self._dist else None)

    def sum(self, value: float) -> float:
        """The sum over the ranks (the work all replicas did)."""
        return self._reduce(value, self._dist.ReduceOp.SUM if self._dist else None)

    def close(self) -> None:
        if self._dist:
            self._dist.destroy_process_group()
            self._dist = None
