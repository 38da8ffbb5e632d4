"""Multi-GPU layout of the all-pairs job: pairs are independent, so each
rank takes its own contiguous batches and no collective touches the data;
the only collectives are a barrier around the timed region and a maximum
of the per-rank times (weak scaling: value = pairs of all ranks / slowest
rank's time).

Batch s of rank r covers pairs [(r*S + s)*B, (r*S + s + 1)*B) of the pair
list, S = steps per rank (warm-up included), B = pairs per step
(``rank_batch``); ``spread_batch`` places the world*S batches evenly over
the whole list instead, so that a sample of steps covers every part of the
all-pairs job (its pairs' rows a run from 0 to N-2).
"""
from __future__ import annotations

import numpy as np


def rank_batch(ab: np.ndarray, rank: int, steps: int, step: int, per_step: int) -> np.ndarray:
    """Pairs of batch `step` of `rank` (a view into `ab`)."""
    off = (rank * steps + step) * per_step
    return ab[off:off + per_step]


def spread_batch(ab: np.ndarray, rank: int, world: int, steps: int, step: int,
                 per_step: int) -> np.ndarray:
    """Batch `step` of `rank` when the world*steps batches of per_step
    consecutive pairs are spread evenly over the pair list (first batch at
    the start, last at the end; disjoint while world*steps*per_step <= len)."""
    g = rank * steps + step
    n = world * steps
    span = max(0, len(ab) - per_step)
    off = 0 if n <= 1 else span * g // (n - 1)
    return ab[off:off + per_step]


def pairs_needed(world: int, steps: int, per_step: int) -> int:
    return world * steps * per_step


def max_over_ranks(value: float, device: str | None = None) -> float:
    """Maximum of `value` over the ranks of the default process group (the
    value itself without one)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def weak_scaling_value(world: int, steps: int, per_step: int, seconds_max: float) -> float:
    """Whole-job pairs/s: every rank's timed pairs over the slowest rank's time."""
    return world * steps * per_step / seconds_max
