"""GPU parity: libsdgpu.so through its C ABI against the oracle.

Bit-exact idx and distances for binary / cosine / euclidean / manhattan and
the SNN weights and graph; pearson and js within 1e-12 relative with a
tie-aware idx check (their Armadillo arithmetic is parity unpinned)."""
import numpy as np
import pytest

from backends import GpuBackend, OracleBackend, load_golden, make_x, normalise_cols, same_bits
from parity_cases import KNOWN_ANSWERS, _knn_equal, check_golden_case

pytestmark = pytest.mark.gpu

CASES, ARR = load_golden()
ENGINES = [1, 2, 3]


@pytest.fixture(scope="module")
def orc():
    return OracleBackend()


@pytest.fixture(scope="module", params=ENGINES, ids=["exact", "screen", "tensor"])
def gpu_engine(request, gpu):
    gpu.set_engine(request.param)
    yield gpu
    gpu.set_engine(0)


@pytest.mark.parametrize("case", CASES, ids=[c["id"] for c in CASES])
def test_gpu_matches_reference_golden(gpu_engine, case):
    check_golden_case(gpu_engine, case, ARR)


@pytest.mark.parametrize("fn", KNOWN_ANSWERS, ids=[f.__name__ for f in KNOWN_ANSWERS])
def test_gpu_known_answers(gpu_engine, fn):
    fn(gpu_engine)


@pytest.mark.parametrize("method", ["binary", "cosine", "euclidean", "manhattan", "pearson", "js",
                                    "covariance"])
def test_gpu_random_vs_oracle(gpu_engine, orc, method):
    rng = np.random.default_rng(11)
    for trial in range(5):
        n = int(rng.integers(40, 400))
        nx, ny = int(rng.integers(5, 160)), int(rng.integers(5, 160))
        dens = float(rng.uniform(0.01, 0.3))
        X, Y = make_x(n, nx, dens, 1000 + trial), make_x(n, ny, dens, 2000 + trial)
        if method == "js":
            X, Y = normalise_cols(X), normalise_cols(Y)
        dists = (True, False) if method in ("binary", "cosine", "pearson", "covariance") else (True,)
        for d in dists:
            k = int(rng.integers(1, 25))
            for args in (dict(X=X, Y=None, include_self=False), dict(X=X, Y=None, include_self=True),
                         dict(X=X, Y=Y, include_self=False)):
                want = orc.knn(args["X"], args["Y"], k=k, method=method, dist=d,
                               include_self=args["include_self"])
                got = gpu_engine.knn(args["X"], args["Y"], k=k, method=method, dist=d,
                                     include_self=args["include_self"])
                assert got[2] == want[2]
                assert _knn_equal(method, d, got[:2], want[:2]), (method, d, trial, args["include_self"])


def test_gpu_engines_agree_bit_for_bit(gpu):
    X = make_x(500, 700, 0.05, 5)
    for method in ("binary", "cosine", "euclidean", "manhattan"):
        gpu.set_engine(1)
        a = gpu.knn(X, k=15, method=method)
        gpu.set_engine(2)
        b = gpu.knn(X, k=15, method=method)
        gpu.set_engine(3)
        c = gpu.knn(X, k=15, method=method)
        assert same_bits(a[0], b[0]) and same_bits(a[1], b[1]), method
        assert same_bits(a[0], c[0]) and same_bits(a[1], c[1]), method
    gpu.set_engine(0)


def test_js_screen_equals_exact_engine(gpu):
    """js on the FP32 screen (engine 2: FP32 G with its bound, exact FP64
    re-rank of the survivors) returns the exact engine's result bit for bit;
    a matrix with values outside the bound's range (1e-40) is searched
    exactly by the same call."""
    X = normalise_cols(make_x(3000, 4000, 0.05, 41))
    Y = normalise_cols(make_x(3000, 2500, 0.05, 42))
    T = X.copy()
    T.data[::97] = 1e-40
    for A, B in ((X, None), (X, Y), (T, None)):
        gpu.set_engine(1)
        a = gpu.knn(A, B, k=20, method="js")
        gpu.set_engine(2)
        b = gpu.knn(A, B, k=20, method="js")
        assert a[2] == b[2]
        assert same_bits(a[0], b[0]) and same_bits(a[1], b[1])
    gpu.set_engine(0)


def test_moment_methods_screen_equals_exact_engine(gpu):
    """pearson and covariance on the FP32 screen (engine 2: the matched-product
    sum in FP32, the exact path's moment formula on it with a rigorous bound,
    exact FP64 re-rank of the survivors) return the exact engine's result bit
    for bit: signed values, a constant column, a near-constant one, dist and
    similarity forms; a matrix with a value beyond 2^50 is searched exactly by
    the same call."""
    X = make_x(1500, 3000, 0.06, 51, signed=True)
    Y = make_x(1500, 2200, 0.06, 52, signed=True)
    X = X.tolil()
    X[:, 7] = 2.5                                   # constant column (zero variance)
    X[:750, 8] = 1.0                                # near-constant pattern
    X = X.tocsc()
    X.sort_indices()
    T = X.copy()
    T.data[::101] = 1e20
    for A, B in ((X, None), (X, Y), (T, None)):
        for method, dists in (("pearson", (True, False)), ("covariance", (True,))):
            for d in dists:
                gpu.set_engine(1)
                a = gpu.knn(A, B, k=20, method=method, dist=d)
                gpu.set_engine(2)
                b = gpu.knn(A, B, k=20, method=method, dist=d)
                assert a[2] == b[2]
                assert same_bits(a[0], b[0]) and same_bits(a[1], b[1]), (method, d)
    gpu.set_engine(0)
