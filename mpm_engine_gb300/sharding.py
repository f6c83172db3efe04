"""Scene-parallel batches on several GPUs: one process per GPU, each owning whole
scenes.

A single scene does not shard without domain decomposition, which the reference
does not have. A batch of independent scenes (the batched forward and the batched
identification workloads) does: every scene lives on exactly one GPU, and nothing
crosses between GPUs while the scenes step. The one collective is the sum of the
gradients of parameters that several scenes share, which is a few numbers per
parameter, once per backward pass.

- `partition` assigns scenes to ranks, balanced by particle count (the work of a
  substep grows with it): longest first, each to the least-loaded rank.
- `ShardedBatch` builds only this rank's scenes and steps them as one BatchSolver.
- `reduce_shared_gradients` sums shared-parameter gradients over the ranks.
- `sharded_throughput` is the whole-job rate: every rank's units over the slowest
  rank's time.
"""
from __future__ import annotations

from typing import Callable, Sequence


def partition(weights: Sequence[float], world: int) -> list[list[int]]:
    """Scene indices per rank. Scenes are taken heaviest first (ties by index), each
    going to the rank with the smallest load so far (ties to the lowest rank). Each
    rank's list comes back in ascending scene order. Deterministic, so every rank
    computes the same assignment without communicating."""
    if world < 1:
        raise ValueError("world must be >= 1")
    loads = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(weights)), key=lambda j: (-float(weights[j]), j)):
        r = min(range(world), key=lambda q: (loads[q], q))
        parts[r].append(i)
        loads[r] += float(weights[i])
    return [sorted(p) for p in parts]


def imbalance(parts: list[list[int]], weights: Sequence[float]) -> float:
    """Largest rank load over the mean rank load (1.0 is a perfect split)."""
    loads = [sum(float(weights[i]) for i in p) for p in parts]
    mean = sum(loads) / max(len(loads), 1)
    return max(loads) / mean if mean > 0 else 1.0


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def reduce_shared_gradients(grads: dict, group=None) -> dict:
    """Sums, in place over all ranks, the gradient tensors of parameters the scenes
    share (e.g. {'E': tensor, 'nu': tensor}); returns the same dict. Without an
    initialised process group it returns the gradients unchanged. The tensors must
    be on the backend's device (CPU for gloo, this rank's GPU for NCCL)."""
    dist = _dist()
    if dist is None or dist.get_world_size(group) == 1:
        return grads
    for key in sorted(grads):
        dist.all_reduce(grads[key], op=dist.ReduceOp.SUM, group=group)
    return grads


def sharded_throughput(local_units: float, local_seconds: float, group=None, device: str = "cpu"):
    """(units per second of the whole job, total units, slowest rank's seconds):
    the sum of every rank's units over the maximum of their timed seconds."""
    dist = _dist()
    if dist is None or dist.get_world_size(group) == 1:
        return local_units / local_seconds, local_units, local_seconds
    import torch
    u = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
    t = torch.tensor([float(local_seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(u.item()) / float(t.item()), float(u.item()), float(t.item())


class ShardedBatch:
    """This rank's share of a batch of scenes, stepped as one BatchSolver.

    `make(i)` builds scene i as a loaded Solver on this rank's device; `weights[i]`
    is its particle count (or any cost proxy). Only the scenes `partition` gives
    this rank are built."""

    def __init__(self, make: Callable[[int], object], weights: Sequence[float], rank: int = 0, world: int = 1):
        from .solver import BatchSolver
        if not 0 <= rank < world:
            raise ValueError("rank must lie in [0, world)")
        self.parts = partition(weights, world)
        self.indices = self.parts[rank]
        self.scenes = [make(i) for i in self.indices]
        self.batch = BatchSolver(self.scenes) if self.scenes else None

    def step(self, dt: float, substeps: int = 1):
        if self.batch is not None:
            self.batch.step(dt, substeps)
        return self

    def particles(self) -> int:
        return sum(int(s.n_particles) for s in self.scenes)


__all__ = ["ShardedBatch", "imbalance", "partition", "reduce_shared_gradients", "sharded_throughput"]
