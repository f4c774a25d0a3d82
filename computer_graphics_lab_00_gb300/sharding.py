"""Tank sharding across GPUs: one process per GPU, no data-path collective.

Tanks are independent, so a batch shards by tank. `partition_tanks` assigns
tanks to ranks by a greedy longest-processing-time rule on particle counts
(each tank, largest first, goes to the least-loaded rank; ties go to the
lower rank), which keeps the largest rank within max(N_t) of the mean.
Each rank then advances its own `BatchSolverGpu` with no exchange between
steps. Only end-of-run statistics are reduced, on the host, in FP64
(`reduce_stats`).

The learned correction trains data-parallel: each rank computes the
gradient of its own batch, the gradients are averaged by one all-reduce
(about 84 KB per Adam step), and every rank applies the same Adam update
(`data_parallel_step`).

A single tank does not shard: that would need a slab decomposition with a
halo exchange every substep, which this package does not implement.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Sequence

import numpy as np


def partition_tanks(counts: Sequence[int], world_size: int) -> list[list[int]]:
    """Tank indices per rank (ascending within a rank)."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    counts = [int(c) for c in counts]
    if any(c < 0 for c in counts):
        raise ValueError("tank particle counts must be non-negative")
    order = sorted(range(len(counts)), key=lambda t: (-counts[t], t))
    load = [0] * world_size
    shards: list[list[int]] = [[] for _ in range(world_size)]
    for t in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        shards[r].append(t)
        load[r] += counts[t]
    return [sorted(s) for s in shards]


def shard_loads(counts: Sequence[int], shards: Sequence[Sequence[int]]) -> list[int]:
    return [int(sum(int(counts[t]) for t in s)) for s in shards]


@dataclass
class TankStats:
    """The FP64 sums one rank contributes for its tanks."""

    particles: int = 0
    compression_sum: float = 0.0   # sum over tanks of particles * mean_compression
    density_sum: float = 0.0       # sum over tanks of particles * mean_density
    kinetic_energy: float = 0.0
    max_density: float = 0.0
    nonfinite: int = 0

    @classmethod
    def from_sph_stats(cls, stats) -> "TankStats":
        out = cls()
        for s in stats:
            n = int(s.particles)
            out.particles += n
            out.compression_sum += n * float(s.mean_compression)
            out.density_sum += n * float(s.mean_density)
            out.kinetic_energy += float(s.kinetic_energy)
            out.max_density = max(out.max_density, float(s.max_density))
            out.nonfinite += int(s.nonfinite)
        return out

    def as_array(self) -> np.ndarray:
        return np.array([self.particles, self.compression_sum, self.density_sum, self.kinetic_energy,
                         self.nonfinite], np.float64)


def reduce_stats(local: TankStats, group=None) -> dict:
    """Whole-batch statistics from every rank's sums (all ranks get them).

    Uses torch.distributed on CPU tensors when a process group is
    initialised, so it runs over gloo as well as next to NCCL.
    """
    import torch
    import torch.distributed as dist

    sums = torch.from_numpy(local.as_array())
    peak = torch.tensor([local.max_density], dtype=torch.float64)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(sums, op=dist.ReduceOp.SUM, group=group)
        dist.all_reduce(peak, op=dist.ReduceOp.MAX, group=group)
    particles, comp, dens, ke, nonfinite = sums.tolist()
    n = max(particles, 1.0)
    return {"particles": int(particles), "mean_compression": comp / n, "mean_density": dens / n,
            "kinetic_energy": ke, "max_density": float(peak.item()), "nonfinite": int(nonfinite)}


def data_parallel_step(gradients: Callable[[], tuple[float, np.ndarray]],
                       apply: Callable[[np.ndarray], None], group=None) -> float:
    """One data-parallel Adam step.

    `gradients()` returns this rank's (loss, gradient) for its own batch,
    both means over the batch; `apply(g)` runs the optimiser with gradient g.
    With equal batches per rank the average of the ranks' means is the mean
    over the global batch. Returns the global mean loss.
    """
    import torch
    import torch.distributed as dist

    loss, grad = gradients()
    g = torch.from_numpy(np.ascontiguousarray(grad, dtype=np.float32))
    l = torch.tensor([loss], dtype=torch.float64)
    if dist.is_available() and dist.is_initialized():
        world = dist.get_world_size(group)
        dist.all_reduce(g, op=dist.ReduceOp.SUM, group=group)
        dist.all_reduce(l, op=dist.ReduceOp.SUM, group=group)
        g /= world
        l /= world
    apply(g.numpy())
    return float(l.item())


class ShardedBatch:
    """This rank's share of a tank set on its GPU.

    `tankset` is a `workloads.TankSet`; the rank's tanks keep their global
    indices in `tanks`. Stepping is local; `stats()` reduces over ranks.
    """

    def __init__(self, tankset, rank: int, world_size: int, device: int = 0):
        from .batch import BatchSolverGpu

        self.tankset = tankset
        self.rank = rank
        self.world_size = world_size
        self.tanks = partition_tanks(tankset.counts, world_size)[rank]
        self.solver = None
        if self.tanks:
            params = [tankset.params[t] for t in self.tanks]
            counts = [tankset.counts[t] for t in self.tanks]
            self.solver = BatchSolverGpu(params, counts, device=device)
            for local, t in enumerate(self.tanks):
                self.solver.upload(local, *tankset.initial_state(t))

    @property
    def particles(self) -> int:
        return int(sum(self.tankset.counts[t] for t in self.tanks))

    def run(self, dt: float, substeps: int) -> None:
        if self.solver is not None:
            self.solver.run(dt, substeps)

    def synchronize(self) -> None:
        if self.solver is not None:
            self.solver.synchronize()

    def local_stats(self) -> TankStats:
        return TankStats.from_sph_stats(self.solver.stats()) if self.solver is not None else TankStats()

    def stats(self, group=None) -> dict:
        return reduce_stats(self.local_stats(), group)

    def close(self) -> None:
        if self.solver is not None:
            self.solver.close()
            self.solver = None
