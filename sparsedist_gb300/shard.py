"""Query-column sharding of sparseKNN across ranks (one process per GPU).

The forward kNN has no state shared between query columns (the reference's
block loop, R/sparseKNN.R:248-294, treats every block independently), so N
ranks each search a contiguous share of the query columns against their own
replica of the reference and no collective touches the data path.  Only the
result rows are gathered at the end (``gather=True``), and only because the
caller asked for the whole matrix on every rank.

The k clamp and the degenerate-column masks are properties of the whole
search, so every rank applies them identically: each runs the full search
over its own columns, with the self-exclusion offset given by its first
column, which is what ``search(X[:, lo:hi], ref, col_offset=lo)`` must do.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(ncol: int, world: int, rank: int):
    """Contiguous, balanced [lo, hi) share of ``ncol`` columns for ``rank``."""
    base, extra = divmod(ncol, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def sharded_knn(X, search, *, world: int, rank: int, group=None, gather: bool = True):
    """Runs ``search(cols_lo, cols_hi) -> (idx, dist)`` on this rank's share.

    ``search`` returns the rows of the kNN result for query columns
    [lo, hi) as (hi - lo, k) arrays (idx 1-based into the reference, NA
    padded).  With ``gather`` the full (ncol, k) result is assembled on every
    rank with torch.distributed.all_gather_object; the shards are disjoint and
    ordered by rank, so the assembled matrix is exactly the single-process
    result."""
    ncol = X.shape[1]
    lo, hi = shard_bounds(ncol, world, rank)
    idx, dist = search(lo, hi)
    if not gather or world == 1:
        return (lo, hi), idx, dist
    import torch.distributed as tdist
    parts = [None] * world
    tdist.all_gather_object(parts, (lo, hi, np.asarray(idx), np.asarray(dist)), group=group)
    parts.sort(key=lambda t: t[0])
    k = max(p[2].shape[1] for p in parts)
    full_idx = np.concatenate([p[2] for p in parts], axis=0)
    full_dist = np.concatenate([p[3] for p in parts], axis=0)
    assert full_idx.shape == (ncol, k)
    return (0, ncol), full_idx, full_dist
