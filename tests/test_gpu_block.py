"""sdg_knn_block: rows [q0, q0 + nq) of a resident self-search, with the
whole search's semantics, equal bit for bit to the corresponding rows of
sdg_knn -- the per-rank call of query-column sharding (sparsedist_gb300/
shard.py) and of the reference's block loop."""
import numpy as np
import pytest

from backends import METHODS, make_x, same_bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method,engine", [("cosine", 1), ("cosine", 2), ("cosine", 3), ("binary", 2),
                                           ("euclidean", 2), ("euclidean", 3), ("manhattan", 1), ("js", 1)])
def test_blocks_reassemble_the_full_search(gpu, method, engine):
    from sparsedist_gb300 import _lib
    X = make_x(400, 300, 0.08, 23)
    A = X.toarray()
    A[:, [5, 150]] = 0
    import scipy.sparse as sp
    X = sp.csc_matrix(A)
    X.eliminate_zeros()
    if method == "js":
        s = np.asarray(X.sum(axis=0)).ravel()
        s[s == 0] = 1
        X = sp.csc_matrix(X.multiply(1.0 / s[None, :]))
    gpu.set_engine(engine)
    full = gpu.knn(X, k=9, method=method, include_self=False)
    res = _lib.Resident(gpu.ctx, X.shape[0], X.shape[1], X.indptr, X.indices, X.data)
    k = 9
    parts_i, parts_d = [], []
    for q0, nq in ((0, 77), (77, 1), (78, 150), (228, 72)):
        idx = np.empty(nq * k, np.int32)
        dst = np.empty(nq * k, np.float64)
        ke, fl = np.zeros(1, np.int32), np.zeros(1, np.int32)
        _lib.check(gpu.lib.sdg_knn_block(gpu.h, res.handle, None, q0, nq, METHODS[method], 1, k,
                                         0, 1, idx.ctypes.data, dst.ctypes.data, 0,
                                         ke.ctypes.data, fl.ctypes.data))
        e = int(ke[0])
        parts_i.append(idx[:nq * e].reshape(e, nq).T)
        parts_d.append(dst[:nq * e].reshape(e, nq).T)
    gpu.set_engine(0)
    res.free()
    assert same_bits(np.concatenate(parts_i), full[0])
    assert same_bits(np.concatenate(parts_d), full[1])
