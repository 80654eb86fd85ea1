"""Dense embedding columns (the 256 x 2,000,000 embedding path): the BF16 screens (mode 0,
the fused tcgen05 kernel, one CTA per 128-query group; mode 3, the same screen on CTA
pairs (cta_group::2 UMMAs of 256 queries) for blocks of more than 128 queries; mode 2, the
cuBLAS slab) with the exact FP64 re-rank
must return the oracle's sparseKNN result on the same data bit for bit (idx
and distances), near-duplicate columns included; the plain FP32 path (mode 1)
is only reported (its recall is not exact)."""
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


@pytest.mark.parametrize("mode", [0, 2, 3])
@pytest.mark.parametrize("method,code", [("cosine", 1), ("euclidean", 2)])
def test_bf16_screen_with_exact_rerank_equals_oracle(method, code, mode):
    import ctypes as C
    import torch
    from sparsedist_gb300 import _lib, synth
    X = synth.dense_embeddings(d=64, n=3000, centres=20, seed=3)      # (n, d)
    ctx = _lib.Context()
    h = C.c_void_p()
    _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), 64, 3000, C.byref(h)))
    got = dense_knn(ctx, h, 0, 3000, code, 15, mode)
    plain = dense_knn(ctx, h, 0, 3000, code, 15, 1)
    ctx.lib.sdg_dense_free(h)
    A = X.double().cpu().numpy().T                                       # d x n
    want = OracleBackend().knn(sp.csc_matrix(A), k=15, method=method)
    assert same_bits(got[0], want[0]) and same_bits(got[1], want[1])
    agree = np.mean(plain[0] == want[0])
    assert agree > 0.5                                                   # reported, not required
    torch.cuda.synchronize()


@pytest.mark.parametrize("k", [10, 20, 30])
@pytest.mark.parametrize("mode", [0, 2, 3])
@pytest.mark.parametrize("method,code", [("cosine", 1), ("euclidean", 2)])
def test_bf16_screen_many_segments_and_zero_columns(method, code, mode, k):
    """70,001 references (three 32,768-reference segments, the last one ragged
    and not a multiple of 128) and a query block that starts mid-matrix; two
    all-zero columns (one query, one reference) are degenerate: the query's row
    is all NA and the reference is never returned.  The oracle's two-matrix
    search with k + 1 neighbours, minus each query's own column, is the
    self-search result.  k = 10, 20, 30 use the fused kernel's 16-, 24- and
    32-long lists."""
    import ctypes as C
    import torch
    from sparsedist_gb300 import _lib, synth
    d, n, q0, nq = 32, 70001, 1000, 300
    X = synth.dense_embeddings(d=d, n=n, centres=50, seed=7)
    X[q0 + 5] = 0.0
    X[40000] = 0.0
    ctx = _lib.Context()
    h = C.c_void_p()
    _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), d, n, C.byref(h)))
    got = dense_knn(ctx, h, q0, nq, code, k, mode)
    ctx.lib.sdg_dense_free(h)
    A = sp.csc_matrix(X.double().cpu().numpy().T)
    wi, wd, _ = OracleBackend().knn(A[:, q0:q0 + nq], A, k=k + 1, method=method)
    for t in range(nq):
        if t == 5:
            assert np.all(got[0][t] == np.iinfo(np.int32).min)
            assert np.all(np.isnan(got[1][t]))
            continue
        keep = wi[t] != q0 + t + 1
        assert same_bits(got[0][t], wi[t][keep][:k]), t
        assert same_bits(got[1][t], wd[t][keep][:k]), t
        assert 40001 not in got[0][t]
    torch.cuda.synchronize()


def dense_query(ctx, D, Q, method, k, mode):
    """sdg_dense_knn_query: Q is a C-contiguous float32 (nq, d) array."""
    from sparsedist_gb300 import _lib
    nq, d = Q.shape
    idx = np.empty(nq * k, np.int32)
    dst = np.empty(nq * k, np.float64)
    ke, fl = np.zeros(1, np.int32), np.zeros(1, np.int32)
    _lib.check(ctx.lib.sdg_dense_knn_query(ctx.handle, D, Q.ctypes.data, d, nq, method, k, mode,
                                           idx.ctypes.data, dst.ctypes.data, 0, ke.ctypes.data,
                                           fl.ctypes.data))
    e = int(ke[0])
    return idx[:nq * e].reshape(e, nq).T.copy(), dst[:nq * e].reshape(e, nq).T.copy()


def as_csc(X):
    """(n, d) embeddings -> the d x n dgCMatrix the reference would receive
    (every value stored, exact zeros dropped as Matrix does)."""
    A = np.ascontiguousarray(X.double().cpu().numpy())
    n, d = A.shape
    M = sp.csc_matrix((A.ravel(), np.tile(np.arange(d, dtype=np.int32), n),
                       np.arange(0, (n + 1) * d, d, dtype=np.int64)), shape=(d, n))
    M.eliminate_zeros()
    return M


@pytest.mark.parametrize("mode", [0, 2, 3])
@pytest.mark.parametrize("method,code", [("cosine", 1), ("euclidean", 2)])
def test_d256_block_equals_oracle(method, code, mode):
    """The target configuration's kernel shape: d = 256 (four 64-row K chunks),
    200,000 references from the embedding generator (Gaussian clusters and
    1 % near duplicates at 1e-6), a 300-query block (a CTA pair and a partial one) from the middle of the
    matrix, k = 20; idx and distances bit for bit against the oracle's
    two-matrix search with k + 1 neighbours minus each query's own column."""
    import ctypes as C
    import torch
    from sparsedist_gb300 import _lib, synth
    d, n, q0, nq, k = 256, 200000, 123456, 300, 20
    X = synth.dense_embeddings(d=d, n=n, seed=5)
    ctx = _lib.Context()
    h = C.c_void_p()
    _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), d, n, C.byref(h)))
    got = dense_knn(ctx, h, q0, nq, code, k, mode)
    ctx.lib.sdg_dense_free(h)
    A = as_csc(X)
    wi, wd, _ = OracleBackend().knn(A[:, q0:q0 + nq], A, k=k + 1, method=method)
    for t in range(nq):
        keep = wi[t] != q0 + t + 1
        assert same_bits(got[0][t], wi[t][keep][:k]), t
        assert same_bits(got[1][t], wd[t][keep][:k]), t
    torch.cuda.synchronize()


@pytest.mark.parametrize("mode", [0, 2, 3])
@pytest.mark.parametrize("method,code", [("cosine", 1), ("euclidean", 2)])
def test_fp32_cut_near_ties_equal_oracle(method, code, mode):
    """Neighbours that the FP32 third cut cannot tell apart: around each of 12
    base columns (d = 256), 400 references at relative offsets from 2^-25
    (a few FP32 ulps, most elements unchanged) to 2^-12 and 3 exact copies, so
    the k-th neighbour of a base column sits among references closer than the
    cut's FP32 allowance, with exact ties (the copies) broken by index.  The base columns are queries of the resident
    matrix; idx and distances bit for bit against the oracle, and the pairs
    valued exactly stay above k per query (the cut kept the near ties)."""
    import ctypes as C
    import torch
    from sparsedist_gb300 import _lib
    rng = np.random.default_rng(17)
    d, nbase, per, k = 256, 12, 400, 20
    base = rng.standard_normal((nbase, d)).astype(np.float32)
    cols = [base]
    for b in range(nbase):
        scale = np.exp2(rng.uniform(-25, -12, per))[:, None]
        cols.append((base[b] * (1 + scale * rng.standard_normal((per, d)))).astype(np.float32))
        cols.append(np.repeat(base[b][None, :], 3, axis=0))
    cols.append(rng.standard_normal((2000, d)).astype(np.float32))
    X = torch.from_numpy(np.ascontiguousarray(np.concatenate(cols))).cuda()
    n = X.shape[0]
    ctx = _lib.Context()
    h = C.c_void_p()
    _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), d, n, C.byref(h)))
    got = dense_knn(ctx, h, 0, nbase, code, k, mode)
    exact_pairs = ctx.stats()["pairs_exact"]
    ctx.lib.sdg_dense_free(h)
    A = as_csc(X)
    wi, wd, _ = OracleBackend().knn(A[:, 0:nbase], A, k=k + 1, method=method)
    for t in range(nbase):
        keep = wi[t] != t + 1
        assert same_bits(got[0][t], wi[t][keep][:k]), t
        assert same_bits(got[1][t], wd[t][keep][:k]), t
    assert exact_pairs >= nbase * k
    torch.cuda.synchronize()


@pytest.mark.parametrize("k,mode", [(10, 0), (10, 3), (10, 2), (1100, 0), (0, 0)])
def test_nonfinite_query_block_fails_and_context_recovers(k, mode):
    """A query block holding a NaN (or an Inf) fails with SDG_E_NONFINITE and
    returns nothing, whatever the path: the fused screen (the build's
    finiteness flag is read with the first chunk's counts), the slab screen,
    the exact rows of k > 1,024, and an argument error (k = 0) found before
    the flag was read; the next query on the same context is exact."""
    import ctypes as C
    import torch
    from sparsedist_gb300 import _lib, synth
    d, n, nq = 64, 5000, 200
    X = synth.dense_embeddings(d=d, n=n, centres=20, seed=11)
    ctx = _lib.Context()
    h = C.c_void_p()
    _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), d, n, C.byref(h)))
    Q = np.ascontiguousarray(synth.dense_embeddings(d=d, n=nq, centres=20, seed=12).cpu().numpy())
    bad = Q.copy()
    bad[57, 3] = np.nan if k != 1100 else np.inf
    with pytest.raises(_lib.SdgError) as ei:
        dense_query(ctx, h, bad, 1, k, mode)
    assert ei.value.code == -2                      # SDG_E_NONFINITE
    got = dense_query(ctx, h, Q, 1, 10, mode)
    ctx.lib.sdg_dense_free(h)
    want = OracleBackend().knn(as_csc(torch.from_numpy(Q)), as_csc(X), k=10, method="cosine")
    assert same_bits(got[0], want[0]) and same_bits(got[1], want[1])
    torch.cuda.synchronize()


@pytest.mark.parametrize("mode", [0, 2])
def test_unit_columns_of_wide_ragged_columns_equal_oracle(mode):
    """The dense unit columns (unit_csc's recurrence, 8 and 32 columns per
    warp): d = 45 (a ragged last 32-row chunk), values spread over 2^-40 ..
    2^40 with 30 % exact zeros and some negative zeros, an all-zero column and
    a one-entry column; then 320,000 columns of d = 8 (the 32-columns-per-warp
    form).  Cosine idx and distances bit for bit against the oracle."""
    import ctypes as C
    import torch
    from sparsedist_gb300 import _lib
    rng = np.random.default_rng(29)
    cases = []
    d, n = 45, 3000
    X = rng.standard_normal((n, d)) * np.exp2(rng.integers(-40, 40, (n, d)))
    X[rng.random((n, d)) < 0.3] = 0.0
    X[rng.random((n, d)) < 0.02] = -0.0
    X[17] = 0.0
    X[18] = 0.0
    X[18, 44] = 3.5
    cases.append((X.astype(np.float32), 0, 300, 10))
    d, n = 8, 320000
    cases.append((rng.standard_normal((n, d)).astype(np.float32), 1000, 64, 5))
    for Xh, q0, nq, k in cases:
        n, d = Xh.shape
        X = torch.from_numpy(np.ascontiguousarray(Xh)).cuda()
        ctx = _lib.Context()
        h = C.c_void_p()
        _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), d, n, C.byref(h)))
        got = dense_knn(ctx, h, q0, nq, 1, k, mode)
        ctx.lib.sdg_dense_free(h)
        A = as_csc(X)
        wi, wd, _ = OracleBackend().knn(A[:, q0:q0 + nq], A, k=k + 1, method="cosine")
        for t in range(nq):
            if q0 + t == 17:
                assert np.all(got[0][t] == np.iinfo(np.int32).min)
                continue
            keep = wi[t] != q0 + t + 1
            assert same_bits(got[0][t], wi[t][keep][:k]), t
            assert same_bits(got[1][t], wd[t][keep][:k]), t
    torch.cuda.synchronize()


@pytest.mark.parametrize("k", [20, 50, 64])
@pytest.mark.parametrize("mode", [0, 2, 3])
@pytest.mark.parametrize("method,code", [("cosine", 1), ("euclidean", 2)])
def test_query_entry_equals_oracle(method, code, mode, k):
    """sdg_dense_knn_query: new query embeddings (host memory, drawn from the
    same generator with another seed, plus exact copies of two reference
    columns and one all-zero query) against a resident 20,001-column
    reference; the oracle's two-matrix sparseKNN(Q, X) bit for bit.  k = 50
    and 64 use the fused kernel's 64-long lists."""
    import ctypes as C
    import torch
    from sparsedist_gb300 import _lib, synth
    d, n, nq = 96, 20001, 300
    X = synth.dense_embeddings(d=d, n=n, centres=40, seed=8)
    Q = synth.dense_embeddings(d=d, n=nq, centres=40, seed=9)
    Q[7] = X[4242]
    Q[8] = X[20000]
    Q[9] = 0.0
    ctx = _lib.Context()
    h = C.c_void_p()
    _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), d, n, C.byref(h)))
    Qh = np.ascontiguousarray(Q.cpu().numpy())
    got = dense_query(ctx, h, Qh, code, k, mode)
    ctx.lib.sdg_dense_free(h)
    want = OracleBackend().knn(as_csc(Q), as_csc(X), k=k, method=method)
    assert same_bits(got[0], want[0]) and same_bits(got[1], want[1])
    assert got[0][7][0] == 4243 and got[0][8][0] == 20001
    assert np.all(got[0][9] == np.iinfo(np.int32).min)
    torch.cuda.synchronize()


def test_dense_server_each_result_alone_and_in_the_mix():
    """The serving loop over a resident dense reference: 30 requests of 1 to
    700 query columns, cosine and euclidean, k in {10, 20, 50}, submitted
    from 6 threads under a budget that admits several at once; each result is
    bit-identical to the same query alone through sdg_dense_knn_query, and a
    sample of requests to the oracle."""
    import concurrent.futures as cf
    import ctypes as C
    import torch
    from sparsedist_gb300 import _lib, synth
    d, n = 128, 30000
    X = synth.dense_embeddings(d=d, n=n, centres=60, seed=12)
    Qall = np.ascontiguousarray(synth.dense_embeddings(d=d, n=6000, centres=60, seed=13).cpu().numpy())
    ctx = _lib.Context()
    h = C.c_void_p()
    _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), d, n, C.byref(h)))
    rng = np.random.default_rng(3)
    reqs, c0 = [], 0
    for r in range(30):
        m = int(np.exp(rng.uniform(0, np.log(700))))
        reqs.append((Qall[c0:c0 + m], ["cosine", "euclidean"][r % 2], int(rng.choice([10, 20, 50]))))
        c0 = (c0 + m) % 5000
    codes = {"cosine": 1, "euclidean": 2}
    want = [dense_query(ctx, h, Q, codes[m], k, 0) for Q, m, k in reqs]
    srv = _lib.Server(ctx, h, workers=2, max_slots=16, mem_budget=8 << 30, dense=True)
    with cf.ThreadPoolExecutor(6) as ex:
        ids = list(ex.map(lambda t: srv.submit_dense(t[0], codes[t[1]], t[2]), reqs))
    for rid, (Q, m, k), (wi, wd) in zip(ids, reqs, want):
        assert srv.wait(rid, 600000)
        gi, gd, _ = srv.result(rid)
        assert same_bits(gi, wi) and same_bits(gd, wd), (m, k, Q.shape)
    orc = OracleBackend()
    for Q, m, k in reqs[:4]:
        oi, od, _ = orc.knn(sp.csc_matrix(Q.astype(np.float64).T), as_csc(X), k=k, method=m)
        gi, gd = dense_query(ctx, h, Q, codes[m], k, 0)
        assert same_bits(gi, oi) and same_bits(gd, od)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["batches"] < len(reqs)
    with pytest.raises(_lib.SdgError):
        srv.submit_dense(Qall[:3], 0, 10)                 # binary: not a dense method
    srv.close()
    ctx.lib.sdg_dense_free(h)
    torch.cuda.synchronize()
