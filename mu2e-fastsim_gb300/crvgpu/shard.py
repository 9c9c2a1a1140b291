"""Event sharding across ranks (one process per GPU).

Events are independent at every stage and every draw is keyed by the event, so results do not depend on how events
are split: rank r of W processes the contiguous event range event_range(n, W, r); the per-rank cluster tables are
merged by concatenation in rank order (the reference's batch emit/merge, no collective on the data path).
"""
from __future__ import annotations

import numpy as np


def event_range(n_events: int, world: int, rank: int):
    """[first, last) of rank `rank` among `world` ranks (contiguous, sizes differ by at most one)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(int(n_events), int(world))
    first = rank * base + min(rank, extra)
    return first, first + base + (1 if rank < extra else 0)


def merge_tables(parts):
    """Concatenate per-rank dicts of equal keys (cluster tables, member tables) in rank order.  Member rows that
    point at cluster rows are re-based so they index the merged cluster table."""
    parts = [p for p in parts if p]
    if not parts:
        return {}
    out = {}
    ncl = 0
    for k in parts[0]:
        if k == "mem_cl":
            chunks = []
            for p in parts:
                chunks.append(np.asarray(p[k]) + ncl)
                ncl += len(np.asarray(p["cl_event"]))
            out[k] = np.concatenate(chunks)
        else:
            out[k] = np.concatenate([np.asarray(p[k]) for p in parts])
    return out
