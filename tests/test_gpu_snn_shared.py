"""sparseSNN(edges = "shared") on the GPU (sdg_snn_graph_shared): the dgCMatrix
slots (p, i, x) equal the oracle's (pinned to the reference's own
snnJaccardShared on the CPU) bit for bit -- on the reference tests' awkward
fixture for every include_self / prune case, on random index matrices with NA
padding and duplicates, and on a real self-search kNN result through the
Python API."""
import numpy as np
import pytest

from backends import make_x

pytestmark = pytest.mark.gpu

NA = np.iinfo(np.int32).min


def gpu_graph(ctx, idx, include_self, prune):
    from sparsedist_gb300 import _lib
    idx = np.asfortranarray(idx, dtype=np.int32)
    n, k = idx.shape
    nnz = np.zeros(1, np.int64)
    _lib.check(ctx.lib.sdg_snn_graph_shared(ctx.handle, idx.ctypes.data, n, k, int(include_self), float(prune),
                                            nnz.ctypes.data, None, None, None))
    m = int(nnz[0])
    p = np.empty(n + 1, np.int32)
    i = np.empty(max(m, 1), np.int32)
    x = np.empty(max(m, 1), np.float64)
    _lib.check(ctx.lib.sdg_snn_graph_shared(ctx.handle, idx.ctypes.data, n, k, int(include_self), float(prune),
                                            nnz.ctypes.data, p.ctypes.data, i.ctypes.data, x.ctypes.data))
    return p, i[:m], x[:m]


def same(a, b):
    return all(np.array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8)) for x, y in zip(a, b))


@pytest.fixture(scope="module")
def ctx():
    from sparsedist_gb300 import _lib
    return _lib.Context()


def test_awkward_fixture(ctx, oracle):
    idx = np.array([[4, 2, NA], [4, 1, NA], [4, 5, 5], [4, 5, 6], [6, NA, NA], [5, NA, NA]], np.int32)
    for inc in (True, False):
        for pr in (0.0, 0.2, 0.25, 0.5, 2 / 3, 1.0):
            assert same(gpu_graph(ctx, idx, inc, pr), oracle.snn_graph_shared(idx, inc, pr)), (inc, pr)


def test_random_index_matrices(ctx, oracle):
    rng = np.random.default_rng(77)
    for t in range(12):
        n, k = int(rng.integers(2, 3000)), int(rng.integers(1, 25))
        idx = rng.integers(1, n + 1, size=(n, k)).astype(np.int32)
        idx[rng.random((n, k)) < 0.1] = NA
        inc, pr = bool(t % 2), float(rng.choice([0.0, 0.05, 0.2, 0.5]))
        assert same(gpu_graph(ctx, idx, inc, pr), oracle.snn_graph_shared(idx, inc, pr)), t


def test_from_a_knn_result_through_the_api(oracle):
    import sparsedist_gb300 as sdg
    X = make_x(300, 2500, 0.05, 9)
    nn = sdg.sparseKNN(X, k=15, method="cosine", verbose=False)
    for pr in (0.0, 1 / 15):
        g = sdg.sparseSNN(nn, prune=pr, edges="shared", verbose=False)
        p, i, x = oracle.snn_graph_shared(nn["idx"], True, pr)
        assert np.array_equal(g.indptr, p) and np.array_equal(g.indices, i)
        assert np.array_equal(g.data.view(np.uint64), x.view(np.uint64))
        # symmetric, no diagonal
        d = (g - g.T)
        assert d.nnz == 0 or np.all(d.data == 0)
        assert np.all(g.diagonal() == 0)


@pytest.mark.parametrize("chunk", ["1", "5000", "100000"])
def test_expansion_in_row_chunks(ctx, oracle, monkeypatch, chunk):
    """The (i, j) keys are expanded, sorted and counted in chunks of whole
    rows when they exceed the chunk size (SDG_SNN_CHUNK_KEYS lowers it; a
    chunk always holds at least one row): the graph must not change."""
    monkeypatch.setenv("SDG_SNN_CHUNK_KEYS", chunk)
    rng = np.random.default_rng(5)
    n, k = 2500, 12
    # a few hub columns shared by many rows make long R(m) lists
    idx = np.where(rng.random((n, k)) < 0.3, rng.integers(1, 30, (n, k)),
                   rng.integers(1, n + 1, (n, k))).astype(np.int32)
    idx[rng.random((n, k)) < 0.05] = NA
    for inc, pr in ((True, 0.0), (False, 1 / 15), (True, 0.3)):
        assert same(gpu_graph(ctx, idx, inc, pr), oracle.snn_graph_shared(idx, inc, pr)), (chunk, inc, pr)


def test_two_call_protocol_reuses_only_an_identical_query(ctx, oracle):
    """The size query's graph serves the fetch only when every argument and
    the idx contents match; otherwise the fetch builds its own."""
    from sparsedist_gb300 import _lib
    rng = np.random.default_rng(8)
    n, k = 400, 6
    idx = np.asfortranarray(rng.integers(1, n + 1, (n, k)).astype(np.int32))
    nnz = np.zeros(1, np.int64)
    _lib.check(ctx.lib.sdg_snn_graph_shared(ctx.handle, idx.ctypes.data, n, k, 1, 0.0, nnz.ctypes.data,
                                            None, None, None))
    other = idx.copy(order="F")
    other[0, 0] = other[0, 0] % n + 1                 # same pointer shape, other contents
    want = oracle.snn_graph_shared(other, True, 0.0)
    m = len(want[2])
    p = np.empty(n + 1, np.int32)
    i = np.empty(max(m, 1), np.int32)
    x = np.empty(max(m, 1), np.float64)
    _lib.check(ctx.lib.sdg_snn_graph_shared(ctx.handle, other.ctypes.data, n, k, 1, 0.0, nnz.ctypes.data,
                                            p.ctypes.data, i.ctypes.data, x.ctypes.data))
    assert int(nnz[0]) == m and same((p, i[:m], x[:m]), want)
    # and the knn-edge graph after a shared size query with the same idx
    _lib.check(ctx.lib.sdg_snn_graph_shared(ctx.handle, idx.ctypes.data, n, k, 1, 0.0, nnz.ctypes.data,
                                            None, None, None))
    wp, wi, wx = oracle.snn_graph(idx, True, 0.0, True)
    p2 = np.empty(n + 1, np.int32)
    i2 = np.empty(len(wx) + 1, np.int32)
    x2 = np.empty(len(wx) + 1, np.float64)
    _lib.check(ctx.lib.sdg_snn_graph(ctx.handle, idx.ctypes.data, n, k, 1, 0.0, 1, nnz.ctypes.data,
                                     p2.ctypes.data, i2.ctypes.data, x2.ctypes.data))
    assert int(nnz[0]) == len(wx) and same((p2, i2[:len(wx)], x2[:len(wx)]), (wp, wi, wx))
