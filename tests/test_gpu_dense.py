"""Dense embedding columns (configuration 3's path): the BF16 tensor-core
screen with the exact FP64 re-rank must return the oracle's sparseKNN result
on the same data bit for bit (idx and distances), near-duplicate columns
included; the plain FP32 path is only reported (its recall is not exact)."""
import numpy as np
import pytest
import scipy.sparse as sp

from backends import OracleBackend, same_bits

pytestmark = pytest.mark.gpu


def dense_knn(ctx, D, q0, nq, method, k, mode):
    from sparsedist_gb300 import _lib
    idx = np.empty(nq * k, np.int32)
    dst = np.empty(nq * k, np.float64)
    ke, fl = np.zeros(1, np.int32), np.zeros(1, np.int32)
    _lib.check(ctx.lib.sdg_dense_knn_block(ctx.handle, D, q0, nq, method, k, mode, idx.ctypes.data,
                                           dst.ctypes.data, 0, ke.ctypes.data, fl.ctypes.data))
    e = int(ke[0])
    return idx[:nq * e].reshape(e, nq).T.copy(), dst[:nq * e].reshape(e, nq).T.copy()


@pytest.mark.parametrize("method,code", [("cosine", 1), ("euclidean", 2)])
def test_bf16_screen_with_exact_rerank_equals_oracle(method, code):
    import ctypes as C
    import torch
    from sparsedist_gb300 import _lib, synth
    X = synth.dense_embeddings(d=64, n=3000, centres=20, seed=3)      # (n, d)
    ctx = _lib.Context()
    h = C.c_void_p()
    _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), 64, 3000, C.byref(h)))
    got = dense_knn(ctx, h, 0, 3000, code, 15, 0)
    plain = dense_knn(ctx, h, 0, 3000, code, 15, 1)
    ctx.lib.sdg_dense_free(h)
    A = X.double().cpu().numpy().T                                       # d x n
    want = OracleBackend().knn(sp.csc_matrix(A), k=15, method=method)
    assert same_bits(got[0], want[0]) and same_bits(got[1], want[1])
    agree = np.mean(plain[0] == want[0])
    assert agree > 0.5                                                   # reported, not required
    torch.cuda.synchronize()
