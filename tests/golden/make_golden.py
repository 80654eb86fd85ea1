"""Generates tests/golden/golden.npz + golden.json: seeded inputs shaped like
the reference's own test fixtures (make_X() = abs(rsparsematrix(60, 12, 0.3))
and friends, tests/testthat/test-sparseKNN.R:7-12, test-sparseKNNCross.R:7-15,
test-sparseDist.R:6-19)
together with the outputs of the reference's OWN kernels (src/sparseDist.cpp,
src/topK.cpp, src/topKRows.cpp, src/snn.cpp compiled unmodified into
oracle/_ref/ by oracle/build.py), driven by the oracle's restatement of the R
orchestration.

R's RNG is not available, so the matrices are drawn with numpy (PCG64) at the
same shapes, densities and value distributions; the expected outputs are the
reference kernels' results on exactly these inputs.

Run where the reference checkout exists (this container):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import Oracle  # noqa: E402


def make_x(n, p, density, seed, binary=False, signed=False):
    rng = np.random.default_rng(seed)
    M = sp.random(n, p, density=density, format="csc", random_state=rng,
                  data_rvs=lambda k: rng.standard_normal(k))
    if not signed:
        M.data = np.abs(M.data)
    if binary:
        M.data[:] = 1.0
    M.eliminate_zeros()
    M.sort_indices()
    return M


def normalise_cols(M):
    M = M.tocsc(copy=True)
    s = np.asarray(M.sum(axis=0)).ravel()
    keep = s > 0
    M = M[:, np.flatnonzero(keep)]
    s = s[keep]
    M = M.multiply(1.0 / s[None, :]).tocsc()
    M.sort_indices()
    return M


def zero_cols(M, cols):
    A = M.toarray()
    A[:, cols] = 0.0
    R = sp.csc_matrix(A)
    R.sort_indices()
    return R


def main():
    ref = Oracle(ref=True)
    arrays, cases = {}, []

    def put_mat(name, M):
        M = sp.csc_matrix(M)
        arrays[name + "_p"] = M.indptr.astype(np.int32)
        arrays[name + "_i"] = M.indices.astype(np.int32)
        arrays[name + "_x"] = M.data.astype(np.float64)
        arrays[name + "_dim"] = np.array(M.shape, np.int32)

    def add(kind, tag, params, X, Y=None, extra=None):
        cid = "c%03d" % len(cases)
        put_mat(cid + "_X", X)
        if Y is not None:
            put_mat(cid + "_Y", Y)
        case = {"id": cid, "kind": kind, "tag": tag, "params": params, "has_Y": Y is not None}
        if kind == "knn":
            idx, dst, flags = ref.knn(X, Y, **params)
            arrays[cid + "_idx"], arrays[cid + "_dist"] = idx, dst
            case["flags"] = flags
        elif kind == "cross":
            (fi, fd), (ri, rd), flags = ref.knn_cross(X, Y, **params)
            arrays.update({cid + "_fidx": fi, cid + "_fdist": fd, cid + "_ridx": ri,
                           cid + "_rdist": rd})
            case["flags"] = flags
        elif kind == "slab":
            arrays[cid + "_D"] = ref.slab(params["method"], X, Y, params["dist"])
        elif kind == "dist":
            arrays[cid + "_D"] = ref.dist_single(params["method"], X, params["full"], params["diag"],
                                                 params["dist"])
        elif kind == "snn":
            idx = extra
            arrays[cid + "_knnidx"] = idx
            arrays[cid + "_w"] = ref.snn_jaccard(idx, params["include_self"])
            p, i, x = ref.snn_graph(idx, params["include_self"], params["prune"],
                                    params["symmetrise"])
            arrays.update({cid + "_gp": p, cid + "_gi": i, cid + "_gx": x})
        cases.append(case)

    X = make_x(60, 12, 0.3, 1)
    X20 = make_x(60, 20, 0.3, 2)
    Xs = make_x(50, 10, 0.3, 9, signed=True)
    P = normalise_cols(make_x(60, 10, 0.3, 5))
    Q = normalise_cols(make_x(60, 7, 0.3, 6))
    Xb, Yb = make_x(300, 80, 0.05, 11, binary=True), make_x(300, 50, 0.05, 12, binary=True)
    Xd = zero_cols(make_x(60, 10, 0.3, 3), [1, 4])
    for m, dists in (("binary", (True, False)), ("cosine", (True, False)),
                     ("euclidean", (True,)), ("manhattan", (True,)),
                     ("pearson", (True, False))):
        for d in dists:
            add("knn", "self k4 %s dist=%s" % (m, d), dict(k=4, method=m, dist=d), X)
            add("knn", "self include_self k3 %s dist=%s" % (m, d),
                dict(k=3, method=m, dist=d, include_self=True), X)
            add("knn", "block_size=3 k5 %s dist=%s" % (m, d),
                dict(k=5, method=m, dist=d, block_size=3), X20)
            add("knn", "signed k4 %s dist=%s" % (m, d), dict(k=4, method=m, dist=d), Xs)
            add("knn", "cross X(60x12)->Y(60x5) %s dist=%s" % (m, d),
                dict(k=3, method=m, dist=d), X, X[:, :5])
            add("cross", "cross 300x80 / 300x50 bs16 %s dist=%s" % (m, d),
                dict(k=7, method=m, dist=d, block_size=16), Xb, Yb)
            add("slab", "slab %s dist=%s" % (m, d), dict(method=m, dist=d), X, X20)
            add("knn", "degenerate cols 2,5 %s dist=%s" % (m, d), dict(k=3, method=m, dist=d), Xd)
    for m in ("euclidean", "manhattan"):
        add("knn", "drop_degenerate=FALSE %s" % m, dict(k=3, method=m, drop_degenerate=False), Xd)
    add("knn", "js self", dict(k=3, method="js"), P)
    add("knn", "js include_self", dict(k=2, method="js", include_self=True), P)
    add("knn", "js cross", dict(k=3, method="js"), P, Q)
    add("cross", "js cross bidirectional", dict(k=4, method="js", block_size=3), P, Q)
    add("slab", "js slab", dict(method="js", dist=True), P, Q)
    add("knn", "k clamp (5 cols, k=99)", dict(k=99, method="binary"), make_x(60, 5, 0.3, 1))
    ties = sp.csc_matrix(np.tile(np.array([[1.0], [0.0], [1.0], [0.0]]), (1, 6)))
    add("knn", "ties euclidean (test-sparseKNN.R:160-168)", dict(k=3, method="euclidean"), ties)
    mt_x = sp.csc_matrix((np.ones(800), (np.tile(np.arange(20), 40), np.repeat(np.arange(40), 20))),
                         shape=(50, 40))
    mt_y = sp.csc_matrix((np.ones(500), (np.tile(np.arange(20), 25), np.repeat(np.arange(25), 20))),
                         shape=(50, 25))
    for bs in (1, 3, 8, 40):
        add("cross", "massive ties bs=%d (test-sparseKNNCross.R:93-104)" % bs,
            dict(k=6, method="binary", block_size=bs), mt_x, mt_y)
    for self_ in (True, False):
        idx, _, _ = ref.knn(X, k=4, method="binary")
        for prune, sym in ((0.0, True), (1 / 15, True), (0.2, False), (0.0, False)):
            add("snn", "snn include_self=%s prune=%.3f sym=%s" % (self_, prune, sym),
                dict(include_self=self_, prune=prune, symmetrise=sym), X, extra=idx)
    # covariance (fastCov2 through the sparseKNN / sparseKNNCross orchestration)
    for tag, params, A, B in (
            ("self k4", dict(k=4), X, None),
            ("self include_self k3 (self value = variance)", dict(k=3, include_self=True), X, None),
            ("block_size=3 k5", dict(k=5, block_size=3), X20, None),
            ("signed k4", dict(k=4), Xs, None),
            ("degenerate cols 2,5", dict(k=3), Xd, None),
            ("cross X(60x12)->Y(60x5)", dict(k=3), X, X[:, :5])):
        add("knn", "covariance " + tag, dict(params, method="covariance"), A, B)
    add("cross", "covariance cross 300x80 / 300x50 bs16", dict(k=7, method="covariance", block_size=16),
        Xb, Yb)
    add("slab", "covariance slab", dict(method="covariance", dist=True), X, X20)
    # single-matrix sparseDist(X): fastJacc / fastCosine / ... / fastCov with full / diag
    for m, dists in (("binary", (True, False)), ("cosine", (True, False)), ("euclidean", (True,)),
                     ("manhattan", (True,)), ("pearson", (True, False)), ("covariance", (True,)),
                     ("js", (True,))):
        mats = (("P", P),) if m == "js" else (("X", X), ("signed", Xs), ("degenerate", Xd))
        for name, A in mats:
            for full in (False, True):
                for diag in (False, True):
                    for d in dists:
                        add("dist", "sparseDist(%s) %s full=%s diag=%s dist=%s" % (name, m, full, diag, d),
                            dict(method=m, full=full, diag=diag, dist=d), A)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "expected_outputs": "reference kernels (oracle/_ref)", "cases": cases}, f,
                  indent=1)
    print(len(cases), "cases")


if __name__ == "__main__":
    main()
