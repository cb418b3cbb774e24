"""Multi-GPU layout of a batch: paths are independent, so a batch is split into contiguous
path-index ranges, one per rank, and the per-rank results are concatenated; no collective is
needed on the data path (the reference shards paths over threads the same way, with one
atomic counter, src/solve.jl:628-709)."""
from __future__ import annotations

import numpy as np


def shard_range(npaths: int, rank: int, world: int):
    """Contiguous [lo, hi) of path indices for `rank` out of `world` (sizes differ by ≤ 1)."""
    if world < 1 or not (0 <= rank < world) or npaths < 0:
        raise ValueError("need world >= 1, 0 <= rank < world, npaths >= 0")
    base, extra = divmod(npaths, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def gather_results(parts):
    """Concatenate per-rank (results, solutions) in rank order."""
    res = np.concatenate([p[0] for p in parts])
    sol = np.concatenate([p[1] for p in parts])
    return res, sol
