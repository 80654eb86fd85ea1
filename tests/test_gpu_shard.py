"""Reference-column sharding and sharded sparseKNNCross on the GPU, with the
ranks emulated one after another in one process (their searches never wait
on each other; the all-gather is replaced by the list of parts): each part
is the library's search of every query against one shard of the reference
(sparsedist_gb300.shard.knn_reference_shard), and merge_topk of the parts
must equal the single-process sparseKNN / sparseKNNCross bit for bit."""
import numpy as np
import pytest
import scipy.sparse as sp

from backends import make_x, normalise_cols, same_bits

pytestmark = pytest.mark.gpu


def _x(method, seed, ncol=257):
    A = make_x(300, ncol, 0.05, seed).toarray()
    A[:, [0, 7, ncol - 1]] = 0                       # degenerate columns in several shards
    X = sp.csc_matrix(A)
    X.eliminate_zeros()
    if method == "binary":
        X.data[:] = 1.0
    if method == "js":
        X = normalise_cols(X)
    return X


CASES = [("cosine", True, False), ("cosine", False, True), ("binary", False, False),
         ("binary", True, True), ("euclidean", True, False), ("manhattan", True, True),
         ("pearson", False, True), ("js", True, False), ("covariance", True, True),
         ("covariance", True, False)]


@pytest.mark.parametrize("method,dist,include_self", CASES)
def test_reference_sharding_merges_to_single_process(method, dist, include_self):
    import sparsedist_gb300 as sdg
    from sparsedist_gb300.shard import (decreasing_for, knn_reference_shard, merge_topk,
                                        shard_bounds, usable_columns)
    X = _x(method, 9)
    n = X.shape[1]
    for k in (1, 12):
        want = sdg.sparseKNN(X, k=k, method=method, dist=dist, include_self=include_self, verbose=False)
        for world in (2, 3, 7):
            spans = [shard_bounds(n, world, r) for r in range(world)]
            usable = sum(usable_columns(X, a, b) for a, b in spans)   # global_count on real ranks
            k_eff = min(k, usable - (0 if include_self else 1))
            parts = [knn_reference_shard(X, a, b, k_eff=k_eff, method=method, dist=dist,
                                         include_self=include_self) for a, b in spans]
            gi, gd = merge_topk(parts, k_eff, decreasing_for(method, dist))
            assert same_bits(gi, np.ascontiguousarray(want["idx"])), (method, k, world)
            assert same_bits(gd, np.ascontiguousarray(want["dist"])), (method, k, world)


@pytest.mark.parametrize("method,dist", [("cosine", True), ("binary", False), ("manhattan", True),
                                         ("covariance", True)])
def test_cross_sharding_merges_to_single_process(method, dist):
    import sparsedist_gb300 as sdg
    from sparsedist_gb300.shard import (decreasing_for, knn_reference_shard, merge_topk,
                                        shard_bounds, usable_columns)
    X, Y = _x(method, 21, 190), _x(method, 22, 75)
    k = 9
    want = sdg.sparseKNNCross(X, Y, k=k, method=method, dist=dist, verbose=False)
    nx = X.shape[1]
    k_fwd = want["forward"]["idx"].shape[1]
    for world in (2, 3):
        spans = [shard_bounds(nx, world, r) for r in range(world)]
        fwd = [sdg.sparseKNN(X[:, a:b], Y, k=k_fwd, method=method, dist=dist, verbose=False)
               for a, b in spans]
        fi = np.concatenate([f["idx"] for f in fwd], axis=0)
        fd = np.concatenate([f["dist"] for f in fwd], axis=0)
        assert same_bits(fi, np.ascontiguousarray(want["forward"]["idx"]))
        assert same_bits(fd, np.ascontiguousarray(want["forward"]["dist"]))
        k_rev = min(k, sum(usable_columns(X, a, b) for a, b in spans))
        parts = [knn_reference_shard(Y, a, b, Y=X, k_eff=k_rev, method=method, dist=dist)
                 for a, b in spans]
        ri, rd = merge_topk(parts, k_rev, decreasing_for(method, dist))
        assert same_bits(ri, np.ascontiguousarray(want["reverse"]["idx"]))
        assert same_bits(rd, np.ascontiguousarray(want["reverse"]["dist"]))
