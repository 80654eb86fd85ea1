"""Single-matrix sparseDist(X) and covariance on the GPU, through the C ABI
(sdg_dist) and the Python API, against the oracle: bit for bit for binary,
cosine, euclidean and manhattan, within 1e-12 relative for pearson, js and
covariance.  Both the resident path (lower triangle + on-device mirror) and
the streamed path (column blocks, SDG_DIST_RESIDENT_BYTES lowered) run."""
import numpy as np
import pytest
import scipy.sparse as sp

from backends import GpuBackend, OracleBackend, make_x, same_bits
from dist_cases import KNOWN_DIST, dist_equal, make_p, random_dist_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    return GpuBackend()


@pytest.fixture(scope="module")
def orc():
    return OracleBackend()


@pytest.mark.parametrize("fn", KNOWN_DIST, ids=[f.__name__ for f in KNOWN_DIST])
def test_gpu_dist_known_answers(gpu, fn):
    fn(gpu)


@pytest.mark.parametrize("resident,engine", [(None, 0), (None, 1), (None, 2), ("0", 0), ("4000", 0)])
def test_gpu_dist_random_vs_oracle(gpu, orc, resident, engine, monkeypatch):
    # engine 1: the per-thread merge kernel; 2: the query-centric kernel for
    # the match-only methods; 0: chosen by column length
    if resident is not None:
        monkeypatch.setenv("SDG_DIST_RESIDENT_BYTES", resident)
    gpu.set_engine(engine)
    n = 0
    try:
        for method, X, full, diag, dist in random_dist_cases(5 if resident is None else 6, 2):
            got = gpu.dist_single(method, X, full, diag, dist)
            want = orc.dist_single(method, X, full, diag, dist)
            assert dist_equal(method, got, want), (method, X.shape, full, diag, dist, resident, engine)
            n += 1
    finally:
        gpu.set_engine(0)
    assert n > 60


@pytest.mark.parametrize("engine", [1, 2])
def test_gpu_dist_larger_than_one_tile_grid(gpu, orc, engine):
    # n not a multiple of 32 across several mirror tiles and more than one
    # 2,048-candidate chunk of the query-centric kernel; long columns too
    gpu.set_engine(engine)
    try:
        for X in (make_x(1000, 2300, 0.02, 3), make_x(3000, 300, 0.3, 4)):
            for method in ("binary", "cosine", "euclidean", "covariance"):
                for full in (False, True):
                    got = gpu.dist_single(method, X, full, True, True)
                    want = orc.dist_single(method, X, full, True, True)
                    assert dist_equal(method, got, want), (method, X.shape, full, engine)
    finally:
        gpu.set_engine(0)


def test_sparse_dist_api_storage_and_values(orc):
    import sparsedist_gb300 as sdg
    X = make_x(60, 8, 0.3, 1)
    # dense for distances, scipy csc for coefficients (test-sparseDist.R:71-77)
    for m, d in (("euclidean", True), ("manhattan", True), ("binary", True)):
        r = sdg.sparseDist(X, method=m, dist=d, verbose=False)
        assert isinstance(r, np.ndarray) and r.shape == (8, 8)
        assert same_bits(np.ascontiguousarray(r), np.ascontiguousarray(orc.dist_single(m, X, False, False, d)))
    for m, d in (("binary", False), ("covariance", True), ("pearson", False), ("cosine", False)):
        r = sdg.sparseDist(X, method=m, dist=d, full=True, diag=True, verbose=False)
        assert sp.issparse(r) and r.shape == (8, 8), m
        want = orc.dist_single(m, X, True, True, d)
        assert dist_equal(m, r.toarray(), want), m
        assert r.nnz == np.count_nonzero(want), m
    # the default call, the jaccard alias, dense input (test-sparseDist.R:21-36, :197-204)
    a = sdg.sparseDist(X, verbose=False)
    assert a.shape == (8, 8)
    assert np.array_equal(sdg.sparseDist(X, method="jaccard", verbose=False), a)
    e = sdg.sparseDist(X, method="euclidean", verbose=False)
    assert np.array_equal(sdg.sparseDist(X.toarray(), method="euclidean", verbose=False), e)
    # the two-matrix form for every method (test-sparseDist.R:79-91)
    for m in ("binary", "euclidean", "manhattan", "pearson", "covariance"):
        assert sdg.sparseDist(X, X[:, :3], method=m, verbose=False).shape == (8, 3), m
    P = make_p()
    assert sdg.sparseDist(P, P[:, :3], method="js", verbose=False).shape == (P.shape[1], 3)
    with pytest.raises(Exception, match="Mismatched"):
        sdg.sparseDist(X, make_x(50, 8, 0.3, 2), method="euclidean", verbose=False)


def test_covariance_knn_api(orc):
    """sparseKNN / sparseKNNCross with method = "covariance": the largest
    covariances, self value = the variance (test-sparseKNN.R:208-226,
    :278-290; test-sparseKNNCross.R:55-66)."""
    import sparsedist_gb300 as sdg
    X = make_x(80, 40, 0.2, 5)
    Y = make_x(80, 25, 0.2, 6)
    got = sdg.sparseKNN(X, k=6, method="covariance", verbose=False)
    idx, dst, _ = orc.knn(X, k=6, method="covariance")
    assert np.array_equal(got["idx"], idx)
    assert np.allclose(got["dist"], dst, rtol=1e-12, atol=0)
    got = sdg.sparseKNN(X, k=40, method="covariance", include_self=True, verbose=False)
    var = X.toarray().var(axis=0, ddof=1)
    for i in range(40):
        at = list(got["idx"][i]).index(i + 1)
        assert abs(got["dist"][i, at] - var[i]) <= 1e-12 * var[i]
    for bs in (1, 7, 64):
        got = sdg.sparseKNNCross(X, Y, k=5, method="covariance", block_size=bs, verbose=False)
        (fi, fd), (ri, rd), _ = orc.knn_cross(X, Y, k=5, method="covariance", block_size=bs)
        f, r = got["forward"], got["reverse"]
        assert np.array_equal(f["idx"], fi) and np.array_equal(r["idx"], ri)
        assert np.allclose(f["dist"], fd, rtol=1e-12) and np.allclose(r["dist"], rd, rtol=1e-12)
