"""Host-side work distribution across ranks (one process per GPU).

A single terrain does not partition: drops migrate across any cut and every
drop-step's cascade reads and writes a 3 x 3 block, so ranks working on one
terrain are independent replicas.  A batch of terrains partitions by
terrain: every terrain's cycles depend on nothing outside it (the batched
kernel gives each terrain the same bits alone or in any batch), so ranks
take disjoint sets of whole terrains and never exchange data.  The only
collective is the final reduction of counters and timings.

  batch_workload(n, seed)      the batched-terrain workload: n terrains,
                               sides log-uniform in [128, 1024], seeds
                               1000 + i, 0.25 drops per cell per cycle
  shard(costs, world_size)     deterministic longest-processing-time split
  rank_terrains(...)           the terrain indices one rank erodes
  aggregate(units, seconds)    whole-job units and max-over-ranks time
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

# batched-terrain workload constants
SIDE_MIN_LOG2 = 7.0
SIDE_MAX_LOG2 = 10.0
DROPS_PER_CELL = 0.25
SEED_BASE = 1000


@dataclass(frozen=True)
class TerrainSpec:
    index: int
    nx: int
    ny: int
    seed: int
    drops: int

    @property
    def cells(self) -> int:
        return self.nx * self.ny


def batch_workload(n: int = 64, seed: int = 3, drops_per_cell: float = DROPS_PER_CELL) -> list[TerrainSpec]:
    """n square terrains with side round(2^U(7, 10)) (powers of two and
    others), terrain i seeded 1000 + i, drops per cycle proportional to area."""
    if n < 0:
        raise ValueError("n must be >= 0")
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        side = int(round(2.0 ** rng.uniform(SIDE_MIN_LOG2, SIDE_MAX_LOG2)))
        out.append(TerrainSpec(i, side, side, SEED_BASE + i, max(1, int(round(drops_per_cell * side * side)))))
    return out


def terrain_cost(t: TerrainSpec) -> float:
    """Relative cost of one cycle of a terrain: its drop-steps (drops x the
    mean drop life, which does not depend on the size) plus the per-cell
    end-of-cycle work."""
    return float(t.drops) * 400.0 + float(t.cells)


def shard(costs, world_size: int) -> list[list[int]]:
    """Split item indices over world_size ranks: items by decreasing cost
    (ties by index) go to the rank with the least load so far (ties by rank).
    Every item lands on exactly one rank; the result depends only on the
    inputs, so every rank computes the same split without communicating."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    costs = [float(c) for c in costs]
    if any(not math.isfinite(c) or c < 0 for c in costs):
        raise ValueError("costs must be finite and >= 0")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world_size
    parts: list[list[int]] = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def rank_terrains(specs: list[TerrainSpec], world_size: int, rank: int) -> list[TerrainSpec]:
    if not 0 <= rank < world_size:
        raise ValueError("rank out of range")
    part = shard([terrain_cost(t) for t in specs], world_size)[rank]
    return [specs[i] for i in part]


def aggregate(units: float, seconds: float, dist=None) -> tuple[float, float]:
    """Whole-job units (summed over ranks) and job time (the slowest rank).
    `dist` is torch.distributed with an initialised process group, or None
    for a single process."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(units), float(seconds)
    import torch
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(u.item()), float(t.item())
