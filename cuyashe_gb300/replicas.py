"""Replicas: one process per GPU, each multiplying its own share of independent
ciphertext pairs or polynomial products.

Every product, tensor and relinearisation is per polynomial, so the path has no
exchange step and no data-path collective. The reference runs one process on
one GPU with process-global state (src/polynomial.h:35-41,
src/cuda_functions.cu:23-38). Across GPUs, each rank owns a context and its own
copy of the evaluation key. The only collectives are host-side bookkeeping: a
barrier around a timed region and the maximum (or sum) of a scalar over ranks.
They run on whatever process group the launcher set up: NCCL on GPUs, gloo on
CPU.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Optional, Sequence, Tuple


@dataclass
class Replica:
    rank: int = 0
    world: int = 1
    local: int = 0
    group: Optional[object] = None  # torch.distributed, when world > 1

    @property
    def is_root(self) -> bool:
        return self.rank == 0


def from_env(backend: str = "nccl") -> Replica:
    """Reads RANK / WORLD_SIZE / LOCAL_RANK (set by torch.distributed.run) and
    joins the process group when there is more than one rank. With `backend`
    "nccl" the rank's GPU (LOCAL_RANK) becomes the current device first."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    rep = Replica(rank=rank, world=world, local=local)
    if backend == "nccl":
        import torch

        torch.cuda.set_device(local)
    if world > 1:
        import torch
        import torch.distributed as dist

        if not dist.is_initialized():
            if backend == "nccl":
                dist.init_process_group("nccl", device_id=torch.device("cuda", local))
            else:
                dist.init_process_group(backend)
        rep.group = dist
    return rep


def shard(total: int, rank: int, world: int) -> Tuple[int, int]:
    """[start, stop) of rank's share of `total` independent units: contiguous,
    disjoint, covering, sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world or total < 0:
        raise ValueError("bad shard request: total=%d rank=%d world=%d" % (total, rank, world))
    base, extra = divmod(total, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard_items(items: Sequence, rep: Replica):
    start, stop = shard(len(items), rep.rank, rep.world)
    return items[start:stop]


def barrier(rep: Replica) -> None:
    if rep.group is not None:
        rep.group.barrier()


def _reduce(rep: Replica, value: float, op_name: str) -> float:
    if rep.group is None:
        return float(value)
    import torch

    dist = rep.group
    on_gpu = dist.get_backend() == "nccl"
    t = torch.tensor([float(value)], dtype=torch.float64, device="cuda" if on_gpu else "cpu")
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op_name))
    return float(t.item())


def max_over_ranks(rep: Replica, value: float) -> float:
    """The slowest rank's time: the job's time for weak-scaled replicas."""
    return _reduce(rep, value, "MAX")


def sum_over_ranks(rep: Replica, value: float) -> float:
    return _reduce(rep, value, "SUM")


def close(rep: Replica) -> None:
    if rep.group is not None:
        rep.group.barrier()
        rep.group.destroy_process_group()
        rep.group = None
