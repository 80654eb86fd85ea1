"""Checks of the single-matrix sparseDist(X) form, shared by the CPU oracle
tests and the GPU tests.

A backend offers ``dist_single(method, X, full, diag, dist)`` returning the
dense n x n matrix that the reference's fastJacc / fastCosine /
fastEuclidean / fastManhattan / fastCorr / fastJS / fastCov fill
(src/sparseDist.cpp), before R's dense-or-sparse return, and ``slab`` for
the two-matrix form.  ``KNOWN_DIST`` restates the literal fixtures of the
reference's tests/testthat/test-sparseDist.R, each citing its test.
"""
from __future__ import annotations

import math

import numpy as np
import pytest
import scipy.sparse as sp

from backends import make_x, same_bits
from parity_cases import PINNED, REL_TOL, TESTTHAT_TOL

METHODS = ["binary", "cosine", "euclidean", "manhattan", "pearson", "js", "covariance"]


def _csc(cols):
    return sp.csc_matrix(np.column_stack([np.asarray(c, float) for c in cols]))


def make_p(n=60, p=8, density=0.3, seed=1):
    """make_P() of test-sparseDist.R:13-19: non-empty columns scaled to sum 1."""
    P = make_x(n, p, density, seed).toarray()
    P = P[:, P.sum(axis=0) > 0]
    return sp.csc_matrix(P / P.sum(axis=0))


def _eq(a, b, tol=TESTTHAT_TOL):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return a.shape == b.shape and bool(np.all(np.abs(a - b) <= tol * np.maximum(1.0, np.abs(b))))


def kd_unit_diagonal(b):
    # test-sparseDist.R:38-52
    X = make_x(60, 8, 0.3, 1)
    for m in ("binary", "pearson"):
        for dg in (True, False):
            s = b.dist_single(m, X, False, dg, False)
            assert np.array_equal(np.diag(s), np.ones(8)), (m, dg)


def kd_zero_diagonal(b):
    # test-sparseDist.R:54-69
    X = make_x(60, 8, 0.3, 1)
    for m in ("binary", "euclidean", "manhattan", "pearson"):
        d = b.dist_single(m, X, True, True, True)
        assert same_bits(np.ascontiguousarray(np.diag(d)), np.zeros(8)), m
    P = make_p()
    d = b.dist_single("js", P, True, True, True)
    assert same_bits(np.ascontiguousarray(np.diag(d)), np.zeros(P.shape[1]))


def kd_full_symmetry(b):
    # test-sparseDist.R:137-151
    X = make_x(60, 8, 0.3, 1)
    lo = np.tril_indices(8, -1)
    up = np.triu_indices(8, 1)
    for m in ("binary", "euclidean", "manhattan", "pearson", "covariance"):
        full = b.dist_single(m, X, True, True, True)
        assert np.array_equal(full, full.T), m
        low = b.dist_single(m, X, False, True, True)
        assert np.all(low[up] == 0), m
        assert np.array_equal(low[lo], full[lo]), m


def kd_agrees_with_base_r(b):
    # test-sparseDist.R:153-195: euclidean / manhattan (dist()), pearson
    # (cor()), covariance (cov()) and jaccard (a direct set computation)
    X = make_x(60, 8, 0.3, 1)
    A = X.toarray()
    diff = A[:, :, None] - A[:, None, :]
    assert _eq(b.dist_single("euclidean", X, True, True), np.sqrt((diff ** 2).sum(axis=0)))
    assert _eq(b.dist_single("manhattan", X, True, True), np.abs(diff).sum(axis=0))
    assert _eq(b.dist_single("pearson", X, True, True, False), np.corrcoef(A, rowvar=False))
    assert _eq(b.dist_single("covariance", X, True, True), np.cov(A, rowvar=False))
    Z = A != 0
    inter = Z.T.astype(float) @ Z
    uni = Z.sum(axis=0)[:, None] + Z.sum(axis=0)[None, :] - inter
    ref = np.where(uni > 0, inter / np.where(uni > 0, uni, 1), 1.0)
    assert _eq(b.dist_single("binary", X, True, True, False), ref)


def kd_js_standard(b):
    # test-sparseDist.R:99-114
    d = b.dist_single("js", _csc([[1, 0], [0, 1]]), True, True)
    assert abs(d[0, 1] - math.sqrt(math.log(2))) <= TESTTHAT_TOL
    assert same_bits(np.float64(d[0, 0]), np.float64(0.0))
    dn = b.dist_single("js", make_p(), True, True)
    assert np.all(dn <= math.sqrt(math.log(2)) + 1e-12) and np.all(dn >= 0)


def kd_js_invalid(b):
    # test-sparseDist.R:116-123
    with pytest.raises(Exception, match="non-negative"):
        b.dist_single("js", _csc([[-1, 2], [3, 4]]))
    with pytest.raises(Exception, match="finite"):
        b.dist_single("js", _csc([[np.nan, 2], [3, 4]]))


def kd_pearson_range(b):
    # test-sparseDist.R:125-135
    X = make_x(60, 8, 0.3, 1)
    d = b.dist_single("pearson", X, True, True)
    assert np.all(d >= 0) and np.all(d <= 2)
    r = b.slab("pearson", X, X[:, :3], True)
    assert np.all(r >= 0)


def kd_degenerate_columns(b):
    # test-sparseDist.R:216-226: an empty and a constant column give no NaN
    A = make_x(60, 8, 0.3, 1).toarray()
    A[:, 0] = 0
    A[:, 1] = 1
    X = sp.csc_matrix(A)
    for m in ("binary", "euclidean", "manhattan", "pearson", "covariance"):
        assert not np.any(np.isnan(b.dist_single(m, X, True, True))), m


def kd_cosine_direct(b):
    # test-sparseDist.R:236-252
    X = make_x(60, 8, 0.3, 1)
    A = X.toarray()
    nrm = np.sqrt((A ** 2).sum(axis=0))
    with np.errstate(divide="ignore", invalid="ignore"):
        ref = (A.T @ A) / np.outer(nrm, nrm)
    ref[~np.isfinite(ref)] = 0
    ref = np.clip(ref, -1, 1)
    np.fill_diagonal(ref, 1)
    assert _eq(b.dist_single("cosine", X, True, True, False), ref)
    assert _eq(b.dist_single("cosine", X, True, True, True), 1 - ref)


def kd_cosine_signed(b):
    # test-sparseDist.R:254-270
    X = make_x(50, 10, 0.3, 9, signed=True)
    sim = b.dist_single("cosine", X, True, True, False)
    assert np.all((sim >= -1) & (sim <= 1))
    dst = b.dist_single("cosine", X, True, True)
    assert np.all((dst >= 0) & (dst <= 2))
    P = _csc([[1, 2], [-1, -2]])
    assert abs(b.dist_single("cosine", P, True, True, False)[0, 1] + 1) <= TESTTHAT_TOL


def kd_cosine_degenerate(b):
    # test-sparseDist.R:272-297
    A = make_x(60, 8, 0.3, 1).toarray()
    A[:, 0] = 0
    X = sp.csc_matrix(A)
    sim = b.dist_single("cosine", X, False, False, False)
    assert np.array_equal(np.diag(sim), np.ones(8)) and not np.any(np.isnan(sim))
    dst = b.dist_single("cosine", X, True, True)
    assert same_bits(np.ascontiguousarray(np.diag(dst)), np.zeros(8))
    D = _csc([[1, 0], [0, 1]])
    assert same_bits(np.float64(b.dist_single("cosine", D, True, True, False)[0, 1]), np.float64(0.0))


def kd_cosine_cross_matches_single(b):
    # test-sparseDist.R:299-308
    X = make_x(60, 8, 0.3, 1)
    full = b.dist_single("cosine", X, True, True, False)
    cross = b.slab("cosine", X, X[:, :4], False)
    assert _eq(cross, full[:, :4])


def kd_cosine_extremes(b):
    # test-sparseDist.R:310-337
    X = _csc([[1e200, 0], [1e200, 0], [1e-200, 0], [1e-200, 0]])
    sim = b.dist_single("cosine", X, True, True, False)
    assert not np.any(np.isnan(sim))
    for (i, j) in ((0, 1), (2, 3), (0, 2)):
        assert abs(sim[i, j] - 1) <= TESTTHAT_TOL
    dst = b.dist_single("cosine", X, True, True)
    assert not np.any(np.isnan(dst)) and np.all((dst >= 0) & (dst <= 2))


def kd_cosine_nonfinite(b):
    # test-sparseDist.R:339-365
    for bad in (np.inf, np.nan):
        with pytest.raises(Exception, match="finite"):
            b.dist_single("cosine", _csc([[bad, 0], [1, 0]]))
    ok = _csc([[1, 0], [0, 1]])
    assert b.dist_single("cosine", ok).shape == (2, 2)


def kd_cosine_empty_conventions(b):
    # test-sparseDist.R:367-389
    X = _csc([[0, 0], [0, 0], [1, 2]])
    for m in ("cosine", "binary"):
        sim = b.dist_single(m, X, True, True, False)
        assert sim[0, 1] == 1 and sim[0, 2] == 0, m
        assert np.array_equal(np.diag(sim), np.ones(3)), m


def kd_covariance_diag(b):
    # R/sparseDist.R:29-32: the covariance diagonal is the column variance,
    # computed only with diag = TRUE (src/sparseDist.cpp:462-469)
    X = make_x(60, 8, 0.3, 1)
    var = X.toarray().var(axis=0, ddof=1)
    on = b.dist_single("covariance", X, True, True)
    off = b.dist_single("covariance", X, True, False)
    assert _eq(np.diag(on), var, REL_TOL)
    assert np.all(np.diag(off) == 0)
    assert np.array_equal(on - np.diag(np.diag(on)), off)


KNOWN_DIST = [kd_unit_diagonal, kd_zero_diagonal, kd_full_symmetry, kd_agrees_with_base_r,
              kd_js_standard, kd_js_invalid, kd_pearson_range, kd_degenerate_columns,
              kd_cosine_direct, kd_cosine_signed, kd_cosine_degenerate,
              kd_cosine_cross_matches_single, kd_cosine_extremes, kd_cosine_nonfinite,
              kd_cosine_empty_conventions, kd_covariance_diag]


def random_dist_cases(seed, trials):
    """Seeded (method, X, full, diag, dist) cases: ragged sizes, empty and
    constant columns, signed values."""
    rng = np.random.default_rng(seed)
    for t in range(trials):
        for method in METHODS:
            n = int(rng.integers(1, 120))
            p = int(rng.integers(1, 70))
            X = make_x(n, p, float(rng.uniform(0.02, 0.4)), 100 * t + 7,
                       signed=(method not in ("js",) and bool(rng.integers(0, 2))))
            if method == "js":
                A = X.toarray()
                s = A.sum(axis=0)
                A[:, s > 0] /= s[s > 0]
                X = sp.csc_matrix(A)
            elif p > 2 and rng.integers(0, 2):
                A = X.toarray()
                A[:, 0] = 0
                A[:, -1] = 1.5
                X = sp.csc_matrix(A)
            for full in (False, True):
                for diag in (False, True):
                    for dist in ((True, False) if method in ("binary", "cosine", "pearson") else (True,)):
                        yield method, X, full, diag, dist


def dist_equal(method, got, want):
    if method in PINNED:
        return same_bits(np.ascontiguousarray(got), np.ascontiguousarray(want))
    a, b = np.asarray(got), np.asarray(want)
    if a.shape != b.shape or not np.array_equal(a == 0, b == 0):
        return False
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    return bool(np.all(np.abs(a[~na] - b[~nb]) <= REL_TOL * np.maximum(1.0, np.abs(b[~nb]))))
