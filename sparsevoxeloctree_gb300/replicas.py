"""Replica launch of the engine's step on several GPUs of one node.

The voxelize -> build -> march path does not shard: one scene's fragment list, octree pool and image live
on one GPU, and the reference renders one scene per device (Octree / OctreeTracer hold one pool each).
Running N GPUs therefore means N independent replicas of the whole step (weak scaling) with no collective
on the data path; the only cross-rank traffic is the timing protocol around the timed region:

  * a barrier before and after the timed steps, so every rank times the same window;
  * the maximum over ranks of each rank's mean step time (the job is as slow as its slowest replica);
  * rank 0 alone writes the result line.

This module holds that protocol so the benchmark and the multi-process CPU tests share one code path
(NCCL on GPUs, gloo on CPU).
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass(frozen=True)
class ReplicaEnv:
    rank: int
    world: int
    local_rank: int

    @property
    def leader(self) -> bool:
        return self.rank == 0

    @property
    def parallelism(self) -> str:
        return f"replicas x{self.world}" if self.world > 1 else "single GPU"


def replica_env(environ=None) -> ReplicaEnv:
    """Rank, world size and local rank from the launcher's environment (torchrun's RANK / WORLD_SIZE /
    LOCAL_RANK); one process on one GPU when they are absent."""
    e = os.environ if environ is None else environ
    env = ReplicaEnv(int(e.get("RANK", "0")), int(e.get("WORLD_SIZE", "1")), int(e.get("LOCAL_RANK", "0")))
    if env.world < 1 or not 0 <= env.rank < env.world or env.local_rank < 0:
        raise ValueError(f"inconsistent replica environment {env}")
    return env


def init(env: ReplicaEnv, backend: str = "nccl") -> None:
    """Joins the process group when there is more than one replica (rendezvous from MASTER_ADDR /
    MASTER_PORT)."""
    if env.world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend, rank=env.rank, world_size=env.world)


def finish(env: ReplicaEnv) -> None:
    if env.world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def barrier(env: ReplicaEnv) -> None:
    if env.world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(env: ReplicaEnv, value: float, device=None) -> float:
    """The largest of every rank's `value` (all ranks receive it)."""
    if env.world == 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather(env: ReplicaEnv, value: int, device=None) -> list:
    """Every rank's integer `value`, in rank order (all ranks receive the list)."""
    if env.world == 1:
        return [int(value)]
    import torch
    import torch.distributed as dist
    t = torch.tensor([int(value)], dtype=torch.int64, device=device)
    out = [torch.zeros_like(t) for _ in range(env.world)]
    dist.all_gather(out, t)
    return [int(x.item()) for x in out]
