"""k above the shared-memory list limit (1,024): the reference accepts any
k >= 1 (src/topK.cpp:72, R/sparseKNN.R:121-125), so the library selects
with lists in device scratch there.  Every result is compared with the
oracle: bit for bit for the pinned methods and the selection kernels, within
1e-12 with a tie-aware idx check for js."""
import numpy as np
import pytest

from backends import OracleBackend, make_x, normalise_cols, same_bits
from parity_cases import _knn_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def orc():
    return OracleBackend()


@pytest.mark.parametrize("method", ["binary", "cosine", "euclidean", "manhattan", "js"])
def test_knn_k2000_matches_oracle(gpu, orc, method):
    X = make_x(180, 2600, 0.06, 71)
    if method == "js":
        X = normalise_cols(X)
    for include_self in (False, True):
        want = orc.knn(X, k=2000, method=method, include_self=include_self)
        got = gpu.knn(X, k=2000, method=method, include_self=include_self)
        assert got[2] == want[2]
        assert got[0].shape == (X.shape[1], 2000)
        assert _knn_equal(method, True, got[:2], want[:2]), (method, include_self)


def test_knn_clamped_above_1024(gpu, orc):
    # k larger than the usable references: clamped to 1,199 (> 1,024), flag set
    X = make_x(150, 1200, 0.08, 72)
    want = orc.knn(X, k=5000, method="cosine")
    got = gpu.knn(X, k=5000, method="cosine")
    assert got[2] == want[2] != 0
    assert got[0].shape == want[0].shape == (1200, 1199)
    assert same_bits(got[0], want[0]) and same_bits(got[1], want[1])


def test_knn_cross_k1500_matches_oracle(gpu, orc):
    X, Y = make_x(160, 1700, 0.07, 73), make_x(160, 1900, 0.07, 74)
    for method in ("binary", "cosine"):
        want = orc.knn_cross(X, Y, k=1500, method=method)
        got = gpu.knn_cross(X, Y, k=1500, method=method)
        assert got[2] == want[2]
        for g, w in zip(got[:2], want[:2]):
            assert same_bits(g[0], w[0]) and same_bits(g[1], w[1]), method


def test_topk_block_k2000(gpu, orc):
    rng = np.random.default_rng(75)
    D = np.round(rng.standard_normal((3000, 40)), 2)        # many ties
    D[rng.random(D.shape) < 0.02] = np.nan
    D[rng.random(D.shape) < 0.01] = np.inf
    self_row = rng.integers(0, 3001, 40).astype(np.int32)
    for dec in (False, True):
        for k in (1025, 2000, 3500):
            wi, wv = orc.topk_block(D, k, dec, self_row)
            gi, gv = gpu.topk_block(D, k, dec, self_row)
            assert same_bits(gi, wi) and same_bits(gv, wv), (dec, k)


def test_topk_rows_accum_k1100_many_rows(gpu, orc):
    # more rows than the wide selection's warps: each warp takes several rows
    rng = np.random.default_rng(76)
    nrow, k = 12000, 1100
    bi = np.full((nrow, k), np.iinfo(np.int32).min, dtype=np.int32, order="F")
    bv = np.full((nrow, k), np.nan, order="F")
    gi, gv = bi.copy(order="F"), bv.copy(order="F")
    off = 0
    for ncol in (700, 900):
        D = np.round(rng.standard_normal((nrow, ncol)), 3)
        D[rng.random(D.shape) < 0.01] = np.nan
        self_col = rng.integers(0, off + ncol + 1, nrow).astype(np.int32)
        bi, bv = orc.topk_rows_accum(D, k, True, bi, bv, off, self_col)
        gi, gv = gpu.topk_rows_accum(D, k, True, gi, gv, off, self_col)
        assert same_bits(gi, bi) and same_bits(gv, bv), ncol
        off += ncol


@pytest.mark.parametrize("method,code", [("cosine", 1), ("euclidean", 2)])
def test_dense_k1100_matches_oracle(orc, method, code):
    # the dense entry above 1,024 neighbours: exact FP64 rows for every query
    import ctypes as C
    import scipy.sparse as sp
    from sparsedist_gb300 import _lib, synth
    from test_gpu_dense import dense_knn
    X = synth.dense_embeddings(d=32, n=1500, centres=10, seed=9)          # (n, d)
    ctx = _lib.Context()
    h = C.c_void_p()
    _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), 32, 1500, C.byref(h)))
    try:
        got = dense_knn(ctx, h, 0, 1500, code, 1100, 0)
    finally:
        ctx.lib.sdg_dense_free(h)
    want = orc.knn(sp.csc_matrix(X.double().cpu().numpy().T), k=1100, method=method)
    assert same_bits(got[0], want[0]) and same_bits(got[1], want[1])
