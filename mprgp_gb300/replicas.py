"""Multi-GPU: replicas only.

QP instances are independent and the MPRGP path has no exchange step, so
several GPUs serve as replicas: one process per GPU, each with its own
context, and no collective on the data path.  A stream of requests is routed
by scene (a follow-up timestep must reach the GPU that holds its scene's
resident A, x and face); the only collectives are the barrier and the
max / sum reductions around the timed region of a measurement.
"""
from __future__ import annotations

import os


def rank_env():
    """(world, rank, local_rank) from the torchrun environment (1, 0, 0 alone)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def route_scene(scene: int, world: int) -> int:
    """The rank that owns a scene (and so serves all of its timesteps)."""
    return scene % world


def split_window(reqs, rank: int, world: int):
    """The requests of a stream that rank `rank` serves: every request of the
    scenes it owns, in arrival order."""
    return [r for r in reqs if route_scene(r.scene, world) == rank]


def _reduce(value: float, op: str) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def max_over_ranks(value: float) -> float:
    return _reduce(value, "max")


def sum_over_ranks(value: float) -> float:
    return _reduce(value, "sum")


def aggregate_throughput(units_per_rank: float, seconds_per_rank: float) -> float:
    """Whole-job throughput of replicas: all ranks' units over the slowest
    rank's time."""
    return sum_over_ranks(units_per_rank) / max_over_ranks(seconds_per_rank)
