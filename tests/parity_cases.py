"""Parity checks shared by the CPU oracle tests and the GPU tests.

* ``check_golden_case``: a backend against the committed outputs of the
  reference's own kernels (tests/golden), bit for bit for the pinned methods
  and within the stated tolerance for pearson / js (Armadillo-dependent,
  parity unpinned).
* ``KNOWN_ANSWERS``: the literal fixtures and known answers of the
  reference's testthat suite, each citing the test it restates.
"""
from __future__ import annotations

import math

import numpy as np
import pytest
import scipy.sparse as sp

from backends import NA_INT, golden_matrix, make_x, same_bits

PINNED = {"binary", "cosine", "euclidean", "manhattan"}
REL_TOL = 1e-12            # plain-path distances: the stated tolerance
TESTTHAT_TOL = 1.5e-8      # testthat's expect_equal() default, where the R test uses it


def _close(a, b, rel=REL_TOL):
    a, b = np.asarray(a), np.asarray(b)
    na_a, na_b = np.isnan(a), np.isnan(b)
    if not np.array_equal(na_a, na_b):
        return False
    fa, fb = a[~na_a], b[~na_b]
    return bool(np.all(np.abs(fa - fb) <= rel * np.maximum(1.0, np.abs(fb))))


def _tie_aware_idx(idx, dist, ref_idx, ref_dist, decreasing, rel=REL_TOL):
    """Every returned neighbour's distance must reach the oracle's k-th
    (bench/R/30-align.R:105-155 style), row by row."""
    for r in range(ref_idx.shape[0]):
        valid = ref_idx[r] != NA_INT
        if (idx[r] != NA_INT).sum() != valid.sum():
            return False
        if valid.sum() == 0:
            continue
        kth = ref_dist[r][valid][-1]
        got = dist[r][idx[r] != NA_INT]
        tol = rel * max(1.0, abs(kth))
        if decreasing and np.any(got < kth - tol):
            return False
        if not decreasing and np.any(got > kth + tol):
            return False
    return True


def _knn_equal(method, dist_flag, got, want):
    gi, gd = got
    wi, wd = want
    if method in PINNED:
        return same_bits(gi, wi) and same_bits(gd, wd)
    dec = (method == "pearson" and not dist_flag) or method == "covariance"
    if same_bits(gi, wi) and _close(gd, wd):
        return True
    return _tie_aware_idx(gi, gd, wi, wd, dec) and gi.shape == wi.shape


def check_golden_case(backend, case, arr):
    cid, kind, p = case["id"], case["kind"], dict(case["params"])
    X = golden_matrix(arr, cid + "_X")
    Y = golden_matrix(arr, cid + "_Y") if case["has_Y"] else None
    if kind == "knn":
        idx, dst, flags = backend.knn(X, Y, **p)
        assert flags == case["flags"], case["tag"]
        assert _knn_equal(p["method"], p.get("dist", True), (idx, dst),
                          (arr[cid + "_idx"], arr[cid + "_dist"])), case["tag"]
    elif kind == "cross":
        (fi, fd), (ri, rd), flags = backend.knn_cross(X, Y, **p)
        assert flags == case["flags"], case["tag"]
        assert _knn_equal(p["method"], p.get("dist", True), (fi, fd),
                          (arr[cid + "_fidx"], arr[cid + "_fdist"])), case["tag"] + " forward"
        assert _knn_equal(p["method"], p.get("dist", True), (ri, rd),
                          (arr[cid + "_ridx"], arr[cid + "_rdist"])), case["tag"] + " reverse"
    elif kind == "slab":
        D = backend.slab(p["method"], X, Y, p["dist"])
        want = arr[cid + "_D"]
        if p["method"] in PINNED:
            assert same_bits(np.ascontiguousarray(D), np.ascontiguousarray(want)), case["tag"]
        else:
            assert _close(D, want), case["tag"]
    elif kind == "dist":
        D = backend.dist_single(p["method"], X, p["full"], p["diag"], p["dist"])
        want = arr[cid + "_D"]
        if p["method"] in PINNED:
            assert same_bits(np.ascontiguousarray(D), np.ascontiguousarray(want)), case["tag"]
        else:
            assert _close(D, want), case["tag"]
    elif kind == "snn":
        idx = arr[cid + "_knnidx"]
        w = backend.snn_jaccard(idx, p["include_self"])
        assert same_bits(w, arr[cid + "_w"]), case["tag"]
        g = backend.snn_graph(idx, p["include_self"], p["prune"], p["symmetrise"])
        assert same_bits(g[0], arr[cid + "_gp"]), case["tag"]
        assert same_bits(g[1], arr[cid + "_gi"]), case["tag"]
        assert same_bits(g[2], arr[cid + "_gx"]), case["tag"]
    else:
        raise AssertionError(kind)


# ---------------------------------------------------------------------------
# known answers from the reference's testthat suite
# ---------------------------------------------------------------------------
def _csc(cols):
    return sp.csc_matrix(np.column_stack([np.asarray(c, float) for c in cols]))


def ka_ties(b):
    # test-sparseKNN.R:160-168: identical columns -> lower index wins
    X = sp.csc_matrix(np.tile(np.array([[1.0], [0], [1], [0]]), (1, 6)))
    idx, dst, _ = b.knn(X, k=3, method="euclidean")
    assert list(idx[3]) == [1, 2, 3]


def ka_na_padding(b):
    # test-sparseKNN.R:182-194: D = c(1, NA, Inf), k = 3 -> one candidate, NA_real_ slots
    from oracle.pyoracle import NA_REAL_BITS
    na = np.array([NA_REAL_BITS], np.uint64).view(np.float64)[0]
    D = np.array([[1.0], [na], [np.inf]])
    idx, dst = b.topk_block(D, 3, False, [0])
    assert idx[0, 0] == 1 and dst[0, 0] == 1.0
    assert idx[0, 1] == NA_INT and idx[0, 2] == NA_INT
    assert dst[0, 1:].view(np.uint64).tolist() == [int(NA_REAL_BITS)] * 2


def ka_signed_zero(b):
    # src/topK.cpp:38-50, 140-148: -0 and +0 compare equal (the tie goes to the
    # lower row) and each slot returns D's own value, sign of zero included
    D = np.array([[-0.0, 1.0], [0.0, -0.0], [1.0, 0.0]])
    for dec, want_i, want_v in ((False, [[1, 2, 3], [2, 3, 1]], [[-0.0, 0.0, 1.0], [-0.0, 0.0, 1.0]]),
                                (True, [[3, 1, 2], [1, 2, 3]], [[1.0, -0.0, 0.0], [1.0, -0.0, 0.0]])):
        idx, dst = b.topk_block(D, 3, dec, [0, 0])
        assert idx.tolist() == want_i, dec
        assert same_bits(dst, np.array(want_v)), dec
    # the running per-row state keeps the sign too (topKRowsAccum)
    bi = np.full((3, 2), NA_INT, np.int32, order="F")
    bv = np.full((3, 2), np.nan, order="F")
    bi, bv = b.topk_rows_accum(D, 2, False, bi, bv, 0, [0, 0, 0])
    assert same_bits(bv, np.array([[-0.0, 1.0], [0.0, -0.0], [0.0, 1.0]])), bv


def ka_topk_validation(b):
    # test-sparseKNN.R:196-206
    D = np.random.default_rng(0).random((3, 2))
    for sr, msg in (([1, 99], "valid 1-based rows"), ([1, -1], "valid 1-based rows")):
        with pytest.raises(Exception, match=msg):
            b.topk_block(D, 2, False, sr)
    with pytest.raises(Exception, match="k must be"):
        b.topk_block(D, 0, False, [0, 0])


def ka_pearson_self(b):
    # test-sparseKNN.R:254-273: constant column's self-correlation restored
    X = _csc([np.ones(5), np.arange(1, 6)])
    idx, dst, _ = b.knn(X, k=2, method="pearson", dist=False, include_self=True)
    at = list(idx[0]).index(1)
    assert dst[0, at] == 1.0
    idx, dst, _ = b.knn(X, k=2, method="pearson", dist=True, include_self=True)
    assert list(idx[:, 0]) == [1, 2] and list(dst[:, 0]) == [0.0, 0.0]


def ka_covariance(b):
    # test-sparseDist.R:169-179: the covariance slab is base R's cov();
    # test-sparseKNN.R:208-226: the largest covariances are the neighbours
    # whatever `dist` says; test-sparseKNN.R:278-290: the self value is the
    # column variance (no restoration).
    X = make_x(60, 10, 0.3, 1)
    D = np.asarray(b.slab("covariance", X, X, True))
    assert np.allclose(D, np.cov(X.toarray(), rowvar=False), rtol=1e-12, atol=1e-15)
    off = D.copy()
    np.fill_diagonal(off, -np.inf)
    want = np.argsort(-off, axis=1, kind="stable")[:, :3] + 1
    for d in (True, False):
        idx, dst, _ = b.knn(X, k=3, method="covariance", dist=d)
        assert np.array_equal(idx, want)
        assert np.all(np.diff(dst, axis=1) <= 0)
    X2 = make_x(60, 6, 0.3, 2)
    idx, dst, _ = b.knn(X2, k=6, method="covariance", include_self=True)
    var = X2.toarray().var(axis=0, ddof=1)
    for i in range(6):
        at = list(idx[i]).index(i + 1)
        assert abs(dst[i, at] - var[i]) <= 1e-12 * var[i]


def ka_js_self(b):
    # test-sparseKNN.R:275-280: exact 0 self-distance for js
    P = make_x(60, 6, 0.3, 1)
    s = np.asarray(P.sum(axis=0)).ravel()
    P = sp.csc_matrix(P.multiply(1.0 / s[None, :]))
    idx, dst, _ = b.knn(P, k=2, method="js", include_self=True)
    assert list(dst[:, 0]) == [0.0] * 6 and list(idx[:, 0]) == list(range(1, 7))


def ka_signed_cancel(b):
    # test-sparseKNN.R:415-433: colSums(abs) decides emptiness, not colSums
    X = _csc([[1, -1, 0, 0], [0, 0, 0, 0], [1, 0, 1, 0], [0, 1, 0, 1]])
    for m in ("euclidean", "cosine"):
        idx, _, _ = b.knn(X, k=2, method=m)
        assert np.all(idx[0] != NA_INT) and np.all(idx[1] == NA_INT)
        assert not np.any(idx[[0, 2, 3]] == 2)
        assert np.any(idx[1:] == 1)


def ka_cross_degenerate(b):
    # test-sparseKNN.R:435-465
    clean = _csc([[1, 0, 1, 0], [0, 1, 0, 1], [1, 1, 0, 0]])
    holed = _csc([[1, 0, 0, 1], [0, 0, 0, 0], [0, 1, 1, 0]])
    a, _, _ = b.knn(holed, clean, k=2)
    assert a.shape == (3, 2) and np.all(a[1] == NA_INT) and np.all((a[[0, 2]] >= 1) & (a[[0, 2]] <= 3))
    bb, _, _ = b.knn(clean, holed, k=2)
    assert np.all(bb != NA_INT) and not np.any(bb == 2)
    cc, _, _ = b.knn(holed, holed, k=2)
    assert np.all(cc[1] == NA_INT) and not np.any(cc == 2)
    d, _, flags = b.knn(clean, holed, k=3)
    assert flags & 1 and d.shape[1] == 2


def ka_k_clamp(b):
    # test-sparseKNN.R:116-121 and :404-413
    X = make_x(60, 5, 0.3, 1)
    idx, _, flags = b.knn(X, k=99)
    assert flags & 1 and idx.shape[1] == 4
    A = make_x(60, 6, 0.3, 1).toarray()
    A[:, :2] = 0
    idx, _, flags = b.knn(sp.csc_matrix(A), k=5)
    assert flags & 1 and idx.shape[1] == 3


def ka_no_candidates(b):
    X = sp.csc_matrix(np.zeros((4, 3)))
    with pytest.raises(Exception, match="No candidate neighbours available"):
        b.knn(X, k=1)


def ka_snn_knowns(b):
    # test-sparseSNN.R:53-57: a row listing itself -> weight 1
    w = b.snn_jaccard(np.array([[1, 1], [2, 2], [3, 3]], np.int32), True)
    assert list(w[:, 1]) == [1.0, 1.0, 1.0]
    # :60-69 disjoint neighbourhoods
    idx = np.array([[2, 3], [1, 4], [1, 3], [2, 4]], np.int32)
    w = b.snn_jaccard(idx, False)
    assert w[0, 0] == 0.0
    # :71-79 NA padding
    idx = np.array([[2, 3], [1, NA_INT], [1, 2]], np.int32)
    w = b.snn_jaccard(idx, True)
    assert np.isnan(w[1, 1])
    # :218-238 include_self overrides explicit self entries: 1/3 vs 0
    idx = np.array([[1, 2], [2, 3], [3, 1]], np.int32)
    assert b.snn_jaccard(idx, True)[0, 1] == 1 / 3
    assert b.snn_jaccard(idx, False)[0, 1] == 0.0
    noself = np.array([[2, NA_INT], [3, NA_INT], [1, NA_INT]], np.int32)
    assert same_bits(b.snn_jaccard(noself, True)[:, 0], b.snn_jaccard(idx, True)[:, 1])
    # :171-179 duplicates keep weight 1, not 2
    p, i, x = b.snn_graph(np.array([[2, 2], [1, 1]], np.int32), True, 0.0, False)
    assert list(x) == [1.0, 1.0]
    # :81-88 out-of-range indices
    for bad in ([[1, 99]], [[1, 0]], [[1, -2]]):
        with pytest.raises(Exception, match="1-based row indices"):
            b.snn_jaccard(np.array(bad, np.int32), True)


def ka_snn_awkward_knn_edges(b):
    # test-sparseSNN-shared.R:26-37 fixture, kNN edge set: 8 undirected
    # off-diagonal edges and node 4's self-loop of weight 1 (:131-141)
    idx = np.array([[4, 2, NA_INT], [4, 1, NA_INT], [4, 5, 5], [4, 5, 6], [6, NA_INT, NA_INT],
                    [5, NA_INT, NA_INT]], np.int32)
    p, i, x = b.snn_graph(idx, True, 0.0, True)
    G = sp.csc_matrix((x, i, p), shape=(6, 6)).toarray()
    off = G.copy()
    np.fill_diagonal(off, 0)
    assert (off != 0).sum() // 2 == 8
    assert G[3, 3] == 1.0


def ka_cosine_extremes(b):
    # test-sparseDist.R:301-328: 1e+-200 magnitudes stay exact
    X = _csc([[1e200, 0], [1e200, 0], [1e-200, 0], [1e-200, 0]])
    D = b.slab("cosine", X, X, False)
    assert abs(D[0, 1] - 1) < TESTTHAT_TOL and abs(D[2, 3] - 1) < TESTTHAT_TOL
    assert abs(D[0, 2] - 1) < TESTTHAT_TOL and not np.any(np.isnan(D))
    # :259-263 antiparallel columns: similarity -1
    P = _csc([[1, 2], [-1, -2]])
    assert abs(b.slab("cosine", P, P, False)[0, 1] + 1) < TESTTHAT_TOL
    # :357-377 empty-column conventions
    E = _csc([[0, 0], [0, 0], [1, 2]])
    S = b.slab("cosine", E, E, False)
    assert S[0, 1] == 1.0 and S[0, 2] == 0.0
    Dd = b.slab("cosine", E, E, True)
    assert Dd[0, 0] == 0.0 and Dd[1, 1] == 0.0 and abs(Dd[2, 2]) < 1e-12


def ka_js_disjoint(b):
    # test-sparseDist.R:101-116: disjoint one-hot columns -> sqrt(log 2)
    P = _csc([[1, 0], [0, 1]])
    D = b.slab("js", P, P, True)
    assert abs(D[0, 1] - math.sqrt(math.log(2))) <= 1e-15 and D[0, 0] == 0.0


def ka_nonfinite(b):
    # test-sparseDist.R:330-355 and :118-125
    inf = _csc([[np.inf, 0], [1, 0]])
    ok = _csc([[1, 0], [0, 1]])
    for m1, m2 in ((inf, inf), (ok, inf), (inf, ok)):
        with pytest.raises(Exception, match="finite"):
            b.slab("cosine", m1, m2, True)
    with pytest.raises(Exception, match="non-negative"):
        b.slab("js", _csc([[-1, 2], [3, 4]]), _csc([[1, 2], [3, 4]]), True)
    with pytest.raises(Exception, match="Mismatched"):
        b.slab("euclidean", make_x(60, 3, 0.3, 1), make_x(50, 3, 0.3, 2), True)


def ka_cross_is_two_knn(b):
    # test-sparseKNNCross.R:18-36 contract on a randomised set
    rng = np.random.default_rng(20240612)
    for trial in range(24):
        nrw = int(rng.integers(40, 161))
        ncx, ncy = int(rng.integers(1, 46)), int(rng.integers(1, 46))
        dens = float(rng.uniform(0.02, 0.25))
        k = int(rng.integers(1, 9))
        bs = int(rng.choice([1, 2, 3, 4, 5, 6, 7, 11, 16, 64]))
        meth = ["binary", "cosine", "euclidean", "manhattan", "pearson", "js", "covariance"][trial % 7]
        dst = bool(rng.integers(0, 2)) if meth in ("binary", "cosine", "pearson") else True
        X = make_x(nrw, ncx, dens, trial * 2)
        Y = make_x(nrw, ncy, dens, trial * 2 + 1)
        if meth == "binary":
            X.data[:] = 1
            Y.data[:] = 1
        try:
            fwd, rev, fl = b.knn_cross(X, Y, k=k, method=meth, dist=dst, block_size=bs)
        except Exception as e:
            assert "No candidate" in str(e)
            continue
        f = b.knn(X, Y, k=k, method=meth, dist=dst, block_size=bs)
        r = b.knn(Y, X, k=k, method=meth, dist=dst, block_size=bs)
        assert same_bits(fwd[0], f[0]) and same_bits(fwd[1], f[1]), (trial, meth)
        assert same_bits(rev[0], r[0]) and same_bits(rev[1], r[1]), (trial, meth)


def ka_block_size_invariance(b):
    # test-sparseKNN.R:50-57 and test-sparseKNNCross.R:68-78
    X = make_x(60, 20, 0.3, 2)
    base = b.knn(X, k=5, block_size=20)
    for bs in (1, 2, 3, 7, 100):
        got = b.knn(X, k=5, block_size=bs)
        assert same_bits(got[0], base[0]) and same_bits(got[1], base[1])
    X = make_x(200, 61, 0.06, 3, binary=True)
    Y = make_x(200, 37, 0.06, 4, binary=True)
    ref = b.knn_cross(X, Y, k=5, method="binary", block_size=61)
    for bs in (1, 2, 7, 13, 60, 61, 62, 1000):
        got = b.knn_cross(X, Y, k=5, method="binary", block_size=bs)
        for u, v in zip(got[0] + got[1], ref[0] + ref[1]):
            assert same_bits(u, v)


def ka_rows_accum_validation(b):
    # src/topKRows.cpp:117-143 messages
    D = np.random.default_rng(1).random((4, 3))
    bi = np.full((4, 2), NA_INT, np.int32, order="F")
    bv = np.full((4, 2), np.nan, order="F")
    with pytest.raises(Exception, match="col_offset must be"):
        b.topk_rows_accum(D, 2, False, bi, bv, -1, [0] * 4)
    with pytest.raises(Exception, match="self_col entries"):
        b.topk_rows_accum(D, 2, False, bi, bv, 0, [0, -1, 0, 0])


KNOWN_ANSWERS = [ka_ties, ka_na_padding, ka_signed_zero, ka_topk_validation, ka_pearson_self, ka_covariance, ka_js_self,
                 ka_signed_cancel, ka_cross_degenerate, ka_k_clamp, ka_no_candidates,
                 ka_snn_knowns, ka_snn_awkward_knn_edges, ka_cosine_extremes, ka_js_disjoint,
                 ka_nonfinite, ka_cross_is_two_knn, ka_block_size_invariance,
                 ka_rows_accum_validation]
