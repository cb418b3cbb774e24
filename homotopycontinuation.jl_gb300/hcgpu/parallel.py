"""Multi-GPU tracking of one batch: paths are independent, so a batch is split into contiguous
path-index ranges, one per device (or per rank), and the per-range results are concatenated
in order; nothing is exchanged while paths are tracked (the reference shards paths over
threads the same way, with one atomic counter, src/solve.jl:628-709).

Two forms:
  * one process, several devices: ``track_on_handles`` drives one library handle per device
    (``EndgameTracker(..., devices=[...])``, ``solve(..., devices=[...])``), one host thread
    each (every blocking library call releases the GIL);
  * one process per device (torchrun): ``sharded_track`` tracks this rank's range and gathers
    every rank's results in rank order with ``torch.distributed.all_gather_object``.
With learned step control, the jump check of the host entry points compares endpoints within
one range only."""
from __future__ import annotations

import threading

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
    """Concatenate per-range result tuples (arrays of equal kind) in range order."""
    return tuple(np.concatenate([p[i] for p in parts]) for i in range(len(parts[0])))


def _renumber(res, lo):
    """Path numbers of a range's records are 1-based within the range; make them global."""
    if res.dtype.names and "path_number" in res.dtype.names:
        res = res.copy()
        res["path_number"] += lo
    return res


def track_on_handles(handles, starts, endgame=True, t1=1.0, t0=0.0):
    """Track ``starts`` split into contiguous ranges over ``handles`` (one per device),
    concurrently; returns (results, solutions, valuation, last points) in path order."""
    starts = np.ascontiguousarray(np.asarray(starts, dtype=np.complex128).reshape(-1, handles[0].n))
    world = len(handles)
    out = [None] * world
    errors = []

    def work(k):
        try:
            lo, hi = shard_range(len(starts), k, world)
            r = handles[k].track(starts[lo:hi], endgame=endgame, t1=t1, t0=t0)
            out[k] = (_renumber(r[0], lo),) + tuple(r[1:])
        except BaseException as e:  # re-raised in the caller's thread
            errors.append(e)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(world)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    if errors:
        raise errors[0]
    return gather_results(out)


_SUMMED = ("paths", "evals_jac", "evals", "evals_dd", "taylor_orders", "lu", "solves", "taylor_fp64_redo",
           "paths_to_fp64", "blocks", "learned_proposals", "learned_rejected", "paths_retracked")


def merge_stats(stats):
    """Counters of several handles' last calls: work counters summed, layout values of the
    first handle (all handles hold the same program)."""
    out = dict(stats[0])
    for k in out:
        if k in _SUMMED or k.startswith("clk_"):
            out[k] = sum(s[k] for s in stats)
    return out


def sharded_track(track_fn, starts, group=None):
    """One process per device: track this rank's contiguous range of ``starts`` with
    ``track_fn(range_starts) -> (results, solutions, ...)`` and return every rank's results
    concatenated in rank order (on every rank). Without an initialised process group this is
    ``track_fn(starts)``."""
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return tuple(track_fn(starts))
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    lo, hi = shard_range(len(starts), rank, world)
    mine = tuple(track_fn(starts[lo:hi]))
    mine = (_renumber(mine[0], lo),) + mine[1:]
    parts = [None] * world
    dist.all_gather_object(parts, mine, group=group)
    return gather_results(parts)
