"""Sharding of the batched form across GPUs: one process per GPU, each stepping its own
contiguous range of independent worlds.  Worlds never exchange data, so the data path
has no collective; only timings (max over ranks) and per-world results are reduced on
the host side.  A single world does not shard (replicas only)."""
from __future__ import annotations

import numpy as np

from .scenes import Scene


def world_ranges(body_counts, world_size: int) -> list:
    """Contiguous [start, end) world ranges, one per rank, balanced by body count (each
    rank takes worlds until its share of the running total is reached)."""
    counts = np.asarray(body_counts, dtype=np.int64)
    nw = len(counts)
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    csum = np.concatenate([[0], np.cumsum(counts)])
    total = csum[-1]
    bounds = [0]
    for r in range(1, world_size):
        target = total * r / world_size
        k = int(np.searchsorted(csum, target, side="left"))
        k = min(max(k, bounds[-1]), nw)
        bounds.append(k)
    bounds.append(nw)
    return [(bounds[r], bounds[r + 1]) for r in range(world_size)]


def bodies_per_world(scene: Scene) -> np.ndarray:
    return np.bincount(scene.bodies["world"], minlength=scene.num_worlds)


def local_scene(scene: Scene, rank: int, world_size: int) -> Scene:
    """The worlds of `rank`, renumbered from 0, as a scene of their own."""
    lo, hi = world_ranges(bodies_per_world(scene), world_size)[rank]
    w = scene.bodies["world"]
    b = scene.bodies[(w >= lo) & (w < hi)].copy()
    b["world"] -= lo
    return Scene(f"{scene.name}[{lo}:{hi}]", b, dt=scene.dt, steps=scene.steps,
                 velocity_iterations=scene.velocity_iterations, position_iterations=scene.position_iterations,
                 num_worlds=hi - lo, seed=scene.seed)


def max_over_ranks(value: float) -> float:
    """Max of a host value over the ranks of the default process group (identity alone)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    backend = dist.get_backend()
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
