"""Sharding across ranks (sparsedist_gb300/shard.py), world size 2 on CPU
with the gloo backend: query columns, reference columns (merge of per-shard
top-k lists) and sparseKNNCross (forward rows sharded, reverse lists merged).

Each rank computes its share of the query columns as the reference's block
loop does (R/sparseKNN.R:248-294: slab of the whole reference against the
block, self-restore / masks, topKBlock), here with the oracle as the
per-rank compute; the gathered result must equal the single-process
sparseKNN bit for bit, for any split.  The GPU version of the per-rank call
(sdg_knn_block) is checked in test_gpu_block.py."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from backends import make_x


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def block_search(orc, X, lo, hi, k, method):
    """Rows [lo, hi) of sparseKNN(X, k, method) the way one iteration of the
    reference's block loop computes them (self-search, include_self = FALSE,
    drop_degenerate = TRUE)."""
    from oracle.pyoracle import NA_REAL_BITS
    na = np.array([NA_REAL_BITS], np.uint64).view(np.float64)[0]
    empty = np.asarray(abs(X).sum(axis=0)).ravel() == 0
    avail = int((~empty).sum()) - 1
    k_eff = min(k, avail)
    D = orc.slab(method, X, X[:, lo:hi], True)          # nref x nb
    D[empty, :] = na
    idx, dst = orc.topk_block(D, k_eff, False, np.arange(lo + 1, hi + 1, dtype=np.int32))
    idx[empty[lo:hi]] = np.int32(-(2 ** 31))
    dst[empty[lo:hi]] = na
    return idx, dst


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.pyoracle import Oracle
    from sparsedist_gb300.shard import sharded_knn
    orc = Oracle()
    X = make_x(80, 53, 0.25, 17)
    A = X.toarray()
    A[:, [3, 30]] = 0                                     # degenerate columns on both shards
    import scipy.sparse as sp
    X = sp.csc_matrix(A)
    X.eliminate_zeros()
    (lo, hi), idx, dst = sharded_knn(X, lambda a, b: block_search(orc, X, a, b, 6, "cosine"),
                                     world=world, rank=rank)
    np.savez(os.path.join(out_dir, "rank%d.npz" % rank), idx=idx, dst=dst, lo=lo, hi=hi)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_query_sharding_matches_single_process(tmp_path):
    port = free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    from oracle.pyoracle import Oracle
    import scipy.sparse as sp
    X = make_x(80, 53, 0.25, 17)
    A = X.toarray()
    A[:, [3, 30]] = 0
    X = sp.csc_matrix(A)
    X.eliminate_zeros()
    want_idx, want_dst, _ = Oracle().knn(X, k=6, method="cosine")
    for r in range(2):
        got = np.load(tmp_path / ("rank%d.npz" % r))
        assert np.array_equal(got["idx"], want_idx)
        assert np.array_equal(got["dst"].view(np.uint64), want_dst.view(np.uint64))


@pytest.mark.parametrize("world", [1, 2, 3, 7])
def test_shard_bounds_cover_exactly(world):
    from sparsedist_gb300.shard import shard_bounds
    for ncol in (1, 5, 53, 1000):
        spans = [shard_bounds(ncol, world, r) for r in range(world)]
        assert spans[0][0] == 0 and spans[-1][1] == ncol
        assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
        sizes = [b - a for a, b in spans]
        assert max(sizes) - min(sizes) <= 1


# ---------------------------------------------------------------------------
# reference-column sharding and the exact merge
# ---------------------------------------------------------------------------
def _na():
    from oracle.pyoracle import NA_REAL_BITS
    return np.array([NA_REAL_BITS], np.uint64).view(np.float64)[0]


def _degenerate_x(seed=17, ncol=53):
    import scipy.sparse as sp
    A = make_x(80, ncol, 0.25, seed).toarray()
    A[:, [3, 30]] = 0
    X = sp.csc_matrix(A)
    X.eliminate_zeros()
    return X


def _empty(M):
    return np.asarray(abs(M).sum(axis=0)).ravel() == 0


def shard_search(orc, Q, R, r0, r1, k_eff, method, dist, decreasing, selfmode):
    """Every query column of Q against reference columns [r0, r1) of R, the
    reference's block-loop body (R/sparseKNN.R:248-294) restricted to that
    shard: slab, masks of degenerate reference columns, topKBlock with the
    self row of the shard, indices made global."""
    D = orc.slab(method, R[:, r0:r1], Q, dist)                 # (r1 - r0) x nq
    D[_empty(R)[r0:r1], :] = _na()
    nq = Q.shape[1]
    sr = np.zeros(nq, np.int32)
    if selfmode:
        q = np.arange(nq)
        inside = (q >= r0) & (q < r1)
        sr[inside] = q[inside] - r0 + 1
    idx, dst = orc.topk_block(D, k_eff, decreasing, sr)
    idx = np.where(idx != np.int32(-(2 ** 31)), idx + r0, idx).astype(np.int32)
    dq = _empty(Q)
    idx[dq] = np.int32(-(2 ** 31))
    dst[dq] = _na()
    return idx, dst


def _rank_ref(rank, world, port, out_dir, method, dist, k):
    import torch.distributed as tdist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.pyoracle import Oracle
    from sparsedist_gb300.shard import global_count, shard_bounds, sharded_knn_reference
    orc = Oracle()
    X = _degenerate_x()
    if method == "binary":
        X.data[:] = 1.0
    decreasing = not dist
    r0, r1 = shard_bounds(X.shape[1], world, rank)
    usable = global_count(int((~_empty(X)[r0:r1]).sum()))      # the one scalar all-reduce
    k_eff = min(k, usable - 1)                                  # self-search, include_self = FALSE
    idx, dst = sharded_knn_reference(
        X.shape[1], lambda a, b: shard_search(orc, X, X, a, b, k_eff, method, dist, decreasing, True),
        k_eff=k_eff, decreasing=decreasing, world=world, rank=rank)
    np.savez(os.path.join(out_dir, "ref%d.npz" % rank), idx=idx, dst=dst)
    tdist.barrier()
    tdist.destroy_process_group()


@pytest.mark.parametrize("method,dist,k", [("cosine", True, 6), ("binary", False, 9), ("euclidean", True, 60)])
def test_two_rank_reference_sharding_matches_single_process(tmp_path, method, dist, k):
    port = free_port()
    mp.spawn(_rank_ref, args=(2, port, str(tmp_path), method, dist, k), nprocs=2, join=True)
    from oracle.pyoracle import Oracle
    X = _degenerate_x()
    if method == "binary":
        X.data[:] = 1.0
    want_idx, want_dst, _ = Oracle().knn(X, k=k, method=method, dist=dist)
    for r in range(2):
        got = np.load(tmp_path / ("ref%d.npz" % r))
        assert np.array_equal(got["idx"], want_idx)
        assert np.array_equal(got["dst"].view(np.uint64), want_dst.view(np.uint64))


def _rank_cross(rank, world, port, out_dir, method, dist, k):
    import torch.distributed as tdist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle.pyoracle import Oracle
    from sparsedist_gb300.shard import global_count, shard_bounds, sharded_knn_cross
    orc = Oracle()
    X = _degenerate_x(21, 47)
    Y = _degenerate_x(22, 31)
    decreasing = not dist
    lo, hi = shard_bounds(X.shape[1], world, rank)
    k_fwd = min(k, int((~_empty(Y)).sum()))                     # Y is whole on every rank
    k_rev = min(k, global_count(int((~_empty(X)[lo:hi]).sum())))

    def forward(a, b):
        Q = X[:, a:b]
        return shard_search(orc, Q, Y, 0, Y.shape[1], k_fwd, method, dist, decreasing, False)

    def reverse(a, b):
        return shard_search(orc, Y, X, a, b, k_rev, method, dist, decreasing, False)

    fwd, rev = sharded_knn_cross(X.shape[1], forward, reverse, k_rev=k_rev, decreasing=decreasing,
                                 world=world, rank=rank)
    np.savez(os.path.join(out_dir, "cross%d.npz" % rank), fi=fwd[0], fd=fwd[1], ri=rev[0], rd=rev[1])
    tdist.barrier()
    tdist.destroy_process_group()


@pytest.mark.parametrize("method,dist,k", [("cosine", True, 5), ("manhattan", True, 8)])
def test_two_rank_cross_sharding_matches_single_process(tmp_path, method, dist, k):
    port = free_port()
    mp.spawn(_rank_cross, args=(2, port, str(tmp_path), method, dist, k), nprocs=2, join=True)
    from oracle.pyoracle import Oracle
    X = _degenerate_x(21, 47)
    Y = _degenerate_x(22, 31)
    (fi, fd), (ri, rd), _ = Oracle().knn_cross(X, Y, k=k, method=method, dist=dist)
    for r in range(2):
        got = np.load(tmp_path / ("cross%d.npz" % r))
        assert np.array_equal(got["fi"], fi) and np.array_equal(got["ri"], ri)
        assert np.array_equal(got["fd"].view(np.uint64), fd.view(np.uint64))
        assert np.array_equal(got["rd"].view(np.uint64), rd.view(np.uint64))


@pytest.mark.parametrize("decreasing", [False, True])
def test_merge_topk_equals_whole_topk(decreasing):
    """Any split of the candidate columns, each part's top k with global
    indices, merges to the whole block's top k (ties, non-finite values,
    short parts, NA padding)."""
    from oracle.pyoracle import Oracle
    from sparsedist_gb300.shard import merge_topk
    orc = Oracle()
    rng = np.random.default_rng(3)
    for trial in range(40):
        nrow, ncol = int(rng.integers(1, 60)), int(rng.integers(1, 9))
        D = np.round(rng.standard_normal((nrow, ncol)), int(rng.integers(0, 3)))   # ties
        D[rng.random((nrow, ncol)) < 0.1] = np.nan
        D[rng.random((nrow, ncol)) < 0.05] = np.inf
        D = np.asfortranarray(D)
        k = int(rng.integers(1, 12))
        want = orc.topk_block(D, k, decreasing, np.zeros(ncol, np.int32))
        cuts = np.sort(rng.integers(0, nrow + 1, int(rng.integers(0, 4))))
        bounds = [0, *cuts.tolist(), nrow]
        parts = []
        for a, b in zip(bounds[:-1], bounds[1:]):
            if b == a:
                continue
            i, d = orc.topk_block(np.asfortranarray(D[a:b]), k, decreasing, np.zeros(ncol, np.int32))
            i = np.where(i != np.int32(-(2 ** 31)), i + a, i).astype(np.int32)
            parts.append((i.reshape(ncol, k), d.reshape(ncol, k)))
        gi, gd = merge_topk(parts, k, decreasing)
        wi, wd = want
        assert np.array_equal(gi, wi.reshape(ncol, k)), trial
        assert np.array_equal(gd.view(np.uint64), wd.reshape(ncol, k).view(np.uint64)), trial
