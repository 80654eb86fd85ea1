"""The serving loop (sdg_server_*): requests of different column counts,
methods and k, submitted concurrently, are admitted by slots and device-memory
budget and packed into shared engine passes; each request's result must be
bit-identical to the same search run alone (sdg_knn_resident), under a
generous budget (many requests in flight, mixed batches) and under a budget
that forces admission one request at a time."""
import concurrent.futures as cf

import numpy as np
import pytest
import scipy.sparse as sp

from backends import METHODS, same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def reference():
    from sparsedist_gb300 import synth
    p, i, x = synth.logcount_csc(nrow=30000, ncol=12000, mean_nnz=1800, seed=11, device="cuda")
    return sp.csc_matrix((x, i, p), shape=(30000, 12000))


def requests(ref, n, seed):
    from sparsedist_gb300 import synth
    rng = np.random.default_rng(seed)
    p, i, x = synth.logcount_csc(nrow=30000, ncol=2000, mean_nnz=1800, seed=seed, device="cuda")
    Q = sp.csc_matrix((x, i, p), shape=(30000, 2000))
    out, c0 = [], 0
    for r in range(n):
        ncol = int(np.exp(rng.uniform(0, np.log(200))))
        ncol = max(1, min(ncol, 2000 - c0))
        method = ["cosine", "binary", "euclidean"][r % 3]
        k = [10, 20, 50][rng.integers(0, 3)]
        out.append((Q[:, c0:c0 + ncol], method, k))
        c0 = (c0 + ncol) % 1800
    return out


def alone(ctx, res, Qm, method, k):
    from sparsedist_gb300 import _lib
    q = _lib.Resident(ctx, Qm.shape[0], Qm.shape[1], Qm.indptr, Qm.indices, Qm.data)
    nq = Qm.shape[1]
    idx = np.empty(nq * k, np.int32)
    dst = np.empty(nq * k, np.float64)
    ke, fl = np.zeros(1, np.int32), np.zeros(1, np.int32)
    _lib.check(ctx.lib.sdg_knn_resident(ctx.handle, q.handle, res.handle, METHODS[method], 1, k, 0, 1,
                                        idx.ctypes.data, dst.ctypes.data, ke.ctypes.data,
                                        fl.ctypes.data))
    q.free()
    e = int(ke[0])
    return idx[:nq * e].reshape(e, nq).T.copy(), dst[:nq * e].reshape(e, nq).T.copy()


@pytest.mark.parametrize("budget,slots", [(64 << 30, 64), (1, 1)])
def test_each_result_is_the_same_alone_and_in_the_mix(reference, budget, slots):
    from sparsedist_gb300 import _lib
    ctx = _lib.Context()
    R = reference
    res = _lib.Resident(ctx, R.shape[0], R.shape[1], R.indptr, R.indices, R.data)
    reqs = requests(R, 24, 5)
    want = [alone(ctx, res, Q, m, k) for Q, m, k in reqs]
    srv = _lib.Server(ctx, res, workers=2, max_slots=slots, mem_budget=budget,
                      methods=[METHODS["cosine"], METHODS["binary"], METHODS["euclidean"]])
    with cf.ThreadPoolExecutor(8) as ex:                 # concurrent arrivals
        ids = list(ex.map(lambda t: srv.submit(t[0].shape[0], t[0].shape[1], t[0].indptr,
                                               t[0].indices, t[0].data, METHODS[t[1]], True, t[2]),
                          reqs))
    for rid, (Q, m, k), (wi, wd) in zip(ids, reqs, want):
        assert srv.wait(rid, 600000)
        gi, gd, fl = srv.result(rid)
        assert same_bits(gi, wi) and same_bits(gd, wd), (m, k, Q.shape)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["p50_s"] <= st["p99_s"]
    if slots == 64:
        assert st["batches"] < len(reqs)                 # requests were packed together
    srv.close()
    res.free()


def test_unprepared_method_is_refused(reference):
    """The workers only read the shared reference: a method whose reference
    data sdg_server_create did not prepare is refused at submit (from any
    number of submitting threads), never prepared lazily by a worker."""
    from sparsedist_gb300 import _lib
    ctx = _lib.Context()
    R = reference[:, :3000]
    res = _lib.Resident(ctx, R.shape[0], R.shape[1], R.indptr, R.indices, R.data)
    srv = _lib.Server(ctx, res, workers=2, max_slots=4, mem_budget=8 << 30, methods=[METHODS["cosine"]])
    Q = R[:, :5]

    def submit(method):
        try:
            srv.submit(Q.shape[0], Q.shape[1], Q.indptr, Q.indices, Q.data, METHODS[method], True, 5)
            return None
        except _lib.SdgError as e:
            return e.code, str(e)

    with cf.ThreadPoolExecutor(2) as ex:
        got = list(ex.map(submit, ["binary", "euclidean", "manhattan", "binary"]))
    for g in got:
        assert g is not None and g[0] == -1 and "not prepared" in g[1]
    rid = srv.submit(Q.shape[0], Q.shape[1], Q.indptr, Q.indices, Q.data, METHODS["cosine"], True, 5)
    assert srv.wait(rid, 600000)
    srv.result(rid)
    srv.close()
    res.free()


def test_cancel_pending_and_admitted_requests(reference):
    """One worker, two slots: the first (large) request runs, the second is
    admitted behind it and the rest wait for a slot.  A cancel that returns
    True must make the request finish with SDG_E_CANCELLED and release it (a
    second result call finds no such request); one that returns False must
    deliver the ordinary result.  Every other request still completes."""
    from sparsedist_gb300 import _lib
    ctx = _lib.Context()
    R = reference
    res = _lib.Resident(ctx, R.shape[0], R.shape[1], R.indptr, R.indices, R.data)
    srv = _lib.Server(ctx, res, workers=1, max_slots=2, mem_budget=64 << 30,
                      methods=[METHODS["cosine"], METHODS["binary"]])
    big = R[:, :2000]
    small = [R[:, 10 * t:10 * t + 7] for t in range(6)]
    first = srv.submit(big.shape[0], big.shape[1], big.indptr, big.indices, big.data, METHODS["cosine"],
                       True, 10)
    ids = [srv.submit(Q.shape[0], Q.shape[1], Q.indptr, Q.indices, Q.data, METHODS["binary"], True, 10)
           for Q in small]
    cancelled = {rid: srv.cancel(rid) for rid in ids[::2]}
    assert any(cancelled.values())          # the waiting requests cannot all have started
    for rid, Q in zip(ids, small):
        assert srv.wait(rid, 600000)
        if cancelled.get(rid):
            with pytest.raises(_lib.SdgError) as e:
                srv.result(rid)
            assert e.value.code == -9
            srv._held[rid] = (Q.shape[1], 10)
            with pytest.raises(_lib.SdgError) as e:
                srv.result(rid)                 # released by the first result call
            assert e.value.code == -1
        else:
            gi, gd, _ = srv.result(rid)
            wi, wd = alone(ctx, res, Q, "binary", 10)
            assert same_bits(gi, wi) and same_bits(gd, wd)
    assert srv.wait(first, 600000)
    srv.result(first)
    srv.close()
    res.free()
