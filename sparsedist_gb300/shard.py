"""Sharding of the kNN searches across ranks (one process per GPU).

* Query columns (``sharded_knn``): the forward kNN has no state shared
  between query columns (the reference's block loop, R/sparseKNN.R:248-294,
  treats every block independently), so N ranks each search a contiguous
  share of the query columns against their own replica of the reference and
  no collective touches the data path.  Only the result rows are gathered at
  the end (``gather=True``), and only because the caller asked for the whole
  matrix on every rank.  The k clamp and the degenerate-column masks are
  properties of the whole search, so every rank applies them identically:
  each runs the full search over its own columns, with the self-exclusion
  offset given by its first column.
* Reference columns (``sharded_knn_reference``), for a reference too large
  to replicate: each rank searches every query against its own share of the
  reference columns and keeps its top k_eff with GLOBAL indices; one
  all-gather of nq * k_eff (index, value) pairs per rank follows, and
  ``merge_topk`` selects the best k_eff under the reference's total order
  (value, then the lower index; src/topK.cpp:38-50).  The top k of a union
  is the top k of the union of each part's top k under a total order, so the
  result is the single-process one bit for bit, whatever the split.  The k
  clamp needs the whole reference's count of usable columns: one all-reduce
  of an integer (``global_count``).
* ``sparseKNNCross`` (``sharded_knn_cross``): with the X columns sharded,
  the forward rows are a query-sharded search; the reverse direction (each
  column of Y against all of X, R/sparseKNNCross.R:133-190, accumulated by
  topKRowsAccum over X blocks) is a reference-sharded search and is merged
  the same way (src/topKRows.cpp:25-30: ties stay exact because the order is
  total).
"""
from __future__ import annotations

import numpy as np

NA_INT = np.int32(-(2 ** 31))
NA_REAL = np.array([0x7FF00000000007A2], np.uint64).view(np.float64)[0]


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
    rank with one tensor all-gather (NCCL on GPUs, gloo on CPUs); the shards
    are disjoint and ordered by rank, so the assembled matrix is exactly the
    single-process result."""
    ncol = X.shape[1]
    lo, hi = shard_bounds(ncol, world, rank)
    idx, dist = search(lo, hi)
    if not gather or world == 1:
        return (lo, hi), idx, dist
    rows = [shard_bounds(ncol, world, r) for r in range(world)]
    parts = _all_gather_lists(np.asarray(idx), np.asarray(dist), [b - a for a, b in rows], group)
    full_idx = np.concatenate([p[0] for p in parts], axis=0)
    full_dist = np.concatenate([p[1] for p in parts], axis=0)
    assert full_idx.shape[0] == ncol
    return (0, ncol), full_idx, full_dist


def merge_topk(parts, k: int, decreasing: bool):
    """Best ``k`` of the candidate lists ``parts`` = [(idx, dist), ...], each
    (nq, k_i) with global 1-based indices and NA padding, under the
    reference's order: value ascending (descending with ``decreasing``), ties
    to the lower index, NA slots last.  Returns (nq, k) int32 / float64 with
    the R NA encodings in unfilled slots."""
    idx = np.concatenate([np.asarray(p[0], np.int32) for p in parts], axis=1)
    val = np.concatenate([np.asarray(p[1], np.float64) for p in parts], axis=1)
    nq, m = idx.shape
    valid = idx != NA_INT
    # non-finite values never enter a top-k list (src/topK.cpp:119), so
    # +inf can stand for "empty slot"
    key = np.where(valid, -val if decreasing else val, np.inf)
    tie = np.where(valid, idx, np.iinfo(np.int32).max)
    order = np.lexsort((tie, key), axis=1)[:, :k]
    out_idx = np.full((nq, k), NA_INT, np.int32)
    out_val = np.full((nq, k), NA_REAL, np.float64)
    w = min(k, m)
    sel_valid = np.take_along_axis(valid, order, axis=1)
    out_idx[:, :w] = np.where(sel_valid, np.take_along_axis(idx, order, axis=1), NA_INT)
    picked = np.take_along_axis(val, order, axis=1)
    out_val[:, :w] = np.where(sel_valid, picked, NA_REAL)
    # np.where keeps NA_REAL's payload only through the float path above;
    # restore the exact bit pattern in the empty slots
    bits = out_val.view(np.uint64)
    bits[:, :w][~sel_valid] = np.uint64(0x7FF00000000007A2)
    return out_idx, out_val


def global_count(local: int, group=None) -> int:
    """Sum of an integer over all ranks (the usable reference columns for the
    k clamp): the one scalar all-reduce of a reference-sharded search."""
    import torch
    import torch.distributed as tdist
    t = torch.tensor([int(local)], dtype=torch.int64)
    if tdist.is_initialized() and tdist.get_world_size(group) > 1:
        tdist.all_reduce(t, op=tdist.ReduceOp.SUM, group=group)
    return int(t.item())


def _all_gather_lists(idx, dist, rows, group):
    """Every rank's (rows[r], k) idx / dist lists on every rank, in rank order.

    One all-gather of a (max(rows), 2k) int64 tensor per rank: idx widened in
    the first k columns, the float64 bit patterns of dist (NA payloads
    included) in the last k.  On an NCCL group the tensors live on the current
    CUDA device; on gloo, on the host.  k is the same on every rank (the
    whole search's clamp), which the lengths exchanged first confirm."""
    import torch
    import torch.distributed as tdist
    idx = np.asarray(idx, np.int32)
    dist = np.ascontiguousarray(np.asarray(dist, np.float64))
    n, k = idx.shape
    dev = torch.device("cuda", torch.cuda.current_device()) if tdist.get_backend(group) == "nccl" \
        else torch.device("cpu")
    world = len(rows)
    ks = [torch.zeros(1, dtype=torch.int64, device=dev) for _ in range(world)]
    tdist.all_gather(ks, torch.tensor([k], dtype=torch.int64, device=dev), group=group)
    if any(int(t.item()) != k for t in ks):
        raise RuntimeError("ranks disagree on k: " + str([int(t.item()) for t in ks]))
    m = max(max(rows), 1)
    buf = np.zeros((m, 2 * k), np.int64)
    buf[:n, :k] = idx
    buf[:n, k:] = dist.view(np.int64)
    mine = torch.from_numpy(buf).to(dev)
    got = [torch.empty_like(mine) for _ in range(world)]
    tdist.all_gather(got, mine, group=group)
    parts = []
    for r, t in enumerate(got):
        a = t.cpu().numpy()[:rows[r]]
        parts.append((a[:, :k].astype(np.int32), np.ascontiguousarray(a[:, k:]).view(np.float64)))
    return parts


def sharded_knn_reference(ncol_ref: int, search_shard, *, k_eff: int, decreasing: bool,
                          world: int, rank: int, group=None):
    """Reference-column sharding: ``search_shard(r0, r1) -> (idx, dist)`` is
    this rank's top ``k_eff`` of every query over reference columns [r0, r1)
    with global 1-based indices (NA padded), computed with the whole search's
    k_eff, masks and self-exclusion.  Returns the merged (nq, k_eff) result on
    every rank."""
    r0, r1 = shard_bounds(ncol_ref, world, rank)
    idx, dist = search_shard(r0, r1)
    if world == 1:
        return merge_topk([(idx, dist)], k_eff, decreasing)
    idx, dist = np.asarray(idx), np.asarray(dist)
    parts = _all_gather_lists(idx, dist, [idx.shape[0]] * world, group)
    return merge_topk(parts, k_eff, decreasing)


def sharded_knn_cross(ncol_x: int, forward_search, reverse_search, *, k_rev: int,
                      decreasing: bool, world: int, rank: int, group=None):
    """sparseKNNCross(X, Y) with the columns of X sharded.

    ``forward_search(lo, hi)`` returns the forward rows for X columns
    [lo, hi) (each an independent query); ``reverse_search(lo, hi)`` returns
    every Y column's top ``k_rev`` over X columns [lo, hi) with global
    indices.  Returns ((fwd_idx, fwd_dist), (rev_idx, rev_dist)), both whole,
    on every rank: forward rows concatenated in rank order, reverse lists
    merged under the total order."""
    lo, hi = shard_bounds(ncol_x, world, rank)
    fi, fd = forward_search(lo, hi)
    ri, rd = reverse_search(lo, hi)
    if world == 1:
        return (np.asarray(fi), np.asarray(fd)), merge_topk([(ri, rd)], k_rev, decreasing)
    rows = [shard_bounds(ncol_x, world, r) for r in range(world)]
    fparts = _all_gather_lists(fi, fd, [b - a for a, b in rows], group)
    ri, rd = np.asarray(ri), np.asarray(rd)
    rparts = _all_gather_lists(ri, rd, [ri.shape[0]] * world, group)
    fwd = (np.concatenate([p[0] for p in fparts], axis=0), np.concatenate([p[1] for p in fparts], axis=0))
    rev = merge_topk(rparts, k_rev, decreasing)
    return fwd, rev


def decreasing_for(method: str, dist: bool) -> bool:
    """R/sparseKNN.R:172-181: similarities and covariance keep the largest."""
    if method == "covariance":
        return True
    return (method in ("binary", "jaccard", "cosine", "pearson")) and not dist


def _self_value(method: str, dist: bool):
    """The exact self value sparseKNN restores with include_self
    (R/sparseKNN.R:265-279); None for covariance, whose computed self value
    (the variance) stands."""
    if method in ("binary", "jaccard", "cosine", "pearson"):
        return 0.0 if dist else 1.0
    if method in ("euclidean", "manhattan", "js"):
        return 0.0
    return None


def knn_reference_shard(X, r0: int, r1: int, *, k_eff: int, Y=None, method="binary", dist=True,
                        include_self=False, drop_degenerate=True, ctx=None):
    """One rank's part of sparseKNN(X, Y) when the reference (Y, or X itself
    in a self-search) is sharded by columns: every column of X against
    reference columns [r0, r1), on this rank's GPU through the library, as
    candidate lists with GLOBAL 1-based indices for ``merge_topk``.

    A self-search is run as a cross search of X against its own shard; the
    self pair is then removed (one extra candidate is asked for, so the
    remaining list is still the shard's top k_eff) and, with include_self,
    re-entered with the exact value sparseKNN restores (covariance keeps its
    computed variance)."""
    import warnings

    import scipy.sparse as sp

    from ._lib import SdgError
    from .api import sparseKNN

    selfmode = Y is None
    R = sp.csc_matrix(X if selfmode else Y)
    Xc = sp.csc_matrix(X)
    nq = Xc.shape[1]
    shard = R[:, r0:r1]
    restore = _self_value(method, dist) if (selfmode and include_self) else None
    keep_computed_self = selfmode and include_self and restore is None
    kk = k_eff + (1 if selfmode else 0)
    try:
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")            # the shard's own k clamp
            res = sparseKNN(Xc, shard, k=kk, method=method, dist=dist,
                            drop_degenerate=drop_degenerate, verbose=False, ctx=ctx)
        idx = np.array(res["idx"], np.int32, copy=True)
        dst = np.array(res["dist"], np.float64, copy=True)
    except SdgError as e:
        if "No candidate" not in str(e):
            raise
        idx = np.full((nq, 0), NA_INT, np.int32)       # no usable column in this shard
        dst = np.full((nq, 0), NA_REAL, np.float64)
    valid = idx != NA_INT
    idx[valid] += r0
    if selfmode and not keep_computed_self:
        me = (np.arange(nq, dtype=np.int64) + 1)[:, None]
        drop = idx == me
        idx[drop] = NA_INT
        dst.view(np.uint64)[drop] = np.uint64(0x7FF00000000007A2)
    if restore is not None:
        q = np.arange(nq)
        owned = (q >= r0) & (q < r1)
        if drop_degenerate:
            owned &= np.asarray(abs(R).sum(axis=0)).ravel() != 0
        si = np.where(owned, q + 1, NA_INT).astype(np.int32)[:, None]
        sv = np.where(owned, restore, NA_REAL)[:, None]
        sv.view(np.uint64)[~owned[:, None]] = np.uint64(0x7FF00000000007A2)
        idx = np.concatenate([idx, si], axis=1)
        dst = np.concatenate([dst, sv], axis=1)
    return idx, dst


def usable_columns(R, r0: int, r1: int, drop_degenerate=True) -> int:
    """Reference columns in [r0, r1) that can be neighbours (not all-zero
    when drop_degenerate, R/sparseKNN.R:214-225): summed over ranks by
    ``global_count`` for the whole search's k clamp."""
    import scipy.sparse as sp
    if not drop_degenerate:
        return r1 - r0
    S = sp.csc_matrix(R)[:, r0:r1]
    return int((np.asarray(abs(S).sum(axis=0)).ravel() != 0).sum())
