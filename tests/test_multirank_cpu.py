"""Query-column sharding across ranks (sparsedist_gb300/shard.py), world size
2 on CPU with the gloo backend.

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
