"""sparseSNN(edges = "shared") on the CPU: the oracle's restatement of
snnJaccardShared (src/snn.cpp:252-447) against the reference's own,
unmodified kernel (oracle/_ref) -- the upper-triangle triplets bit for bit,
in the kernel's order -- and against the known answers of the reference's
tests/testthat/test-sparseSNN-shared.R on its awkward fixture (NA padding, a
duplicate neighbour, an explicit self index, sets of different sizes)."""
import numpy as np
import pytest
import scipy.sparse as sp

NA = np.iinfo(np.int32).min


def awkward_idx():
    return np.array([[4, 2, NA], [4, 1, NA], [4, 5, 5], [4, 5, 6], [6, NA, NA], [5, NA, NA]], np.int32)


def ref_sets(idx, include_self):
    out = []
    for i in range(idx.shape[0]):
        s = {int(v) - 1 for v in idx[i] if v != NA and v - 1 != i}
        if include_self:
            s.add(i)
        out.append(s)
    return out


def ref_shared(idx, include_self=True, prune=0.0):
    """Every pair sharing a neighbour, weighted by the true union, O(n^2)
    straight from the definition (the reference test's ref_shared)."""
    n = idx.shape[0]
    sets = ref_sets(idx, include_self)
    out = np.zeros((n, n))
    for i in range(n - 1):
        for j in range(i + 1, n):
            a, b = sets[i], sets[j]
            if not a or not b:
                continue
            inter = len(a & b)
            if inter == 0:
                continue
            w = inter / len(a | b)
            if w > prune:
                out[i, j] = out[j, i] = w
    return out


def dense(g, n):
    p, i, x = g
    return sp.csc_matrix((x, i, p), shape=(n, n)).toarray()


@pytest.mark.parametrize("include_self", [True, False])
@pytest.mark.parametrize("prune", [0.0, 0.2, 0.5])
def test_shared_weights_match_direct_set_computation(oracle, include_self, prune):
    idx = awkward_idx()
    got = dense(oracle.snn_graph_shared(idx, include_self, prune), 6)
    assert np.array_equal(got, ref_shared(idx, include_self, prune))


def test_shared_structure(oracle):
    m = dense(oracle.snn_graph_shared(awkward_idx(), True, 0.0), 6)
    assert (m != 0).sum() / 2 == 11
    assert np.array_equal(m, m.T)
    assert np.all(np.diag(m) == 0)
    assert m[4, 5] == 1.0                    # N(5) == N(6) == {5, 6}
    assert m[0, 2] == 0.2                    # N(1), N(3) share only node 4 of five


def test_knn_off_diagonal_edges_are_contained_in_shared(oracle):
    idx = awkward_idx()
    knn = dense(oracle.snn_graph(idx, True, 0.0, True), 6)
    shr = dense(oracle.snn_graph_shared(idx, True, 0.0), 6)
    off = lambda m: m - np.diag(np.diag(m))
    assert np.all(off(shr)[off(knn) != 0] != 0)
    assert (off(shr) != 0).sum() > (off(knn) != 0).sum()
    assert (off(knn) != 0).sum() / 2 == 8
    assert knn[3, 3] == 1.0 and np.all(np.diag(shr) == 0)
    both = (off(knn) != 0) & (off(shr) != 0)
    assert np.array_equal(off(knn)[both], off(shr)[both])


@pytest.mark.parametrize("prune", [0.0, 0.2, 0.25, 0.5, 2 / 3])
def test_in_kernel_pruning_matches_pruning_after(oracle, prune):
    idx = awkward_idx()
    full = dense(oracle.snn_graph_shared(idx, True, 0.0), 6)
    want = full.copy()
    want[want <= prune] = 0
    assert np.array_equal(dense(oracle.snn_graph_shared(idx, True, prune), 6), want)


def test_prune_one_is_empty(oracle):
    p, i, x = oracle.snn_graph_shared(awkward_idx(), True, 1.0)
    assert len(i) == 0 and len(p) == 7 and np.all(p == 0)


def test_shared_index_range_error(oracle):
    from oracle.pyoracle import OracleError
    idx = awkward_idx()
    idx[0, 0] = 7
    with pytest.raises(OracleError, match="1-based row indices"):
        oracle.snn_graph_shared(idx, True, 0.0)


def test_shared_bit_identical_to_reference_build(oracle, ref_oracle):
    rng = np.random.default_rng(31)
    cases = [(awkward_idx(), inc, pr) for inc in (True, False) for pr in (0.0, 0.2, 0.5)]
    for t in range(30):
        n, k = int(rng.integers(2, 400)), int(rng.integers(1, 16))
        idx = rng.integers(1, n + 1, size=(n, k)).astype(np.int32)
        idx[rng.random((n, k)) < 0.1] = NA
        cases.append((idx, bool(t % 2), float(rng.choice([0.0, 0.05, 0.2, 0.5]))))
    for idx, inc, pr in cases:
        a = oracle.snn_shared(idx, inc, pr)
        b = ref_oracle.snn_shared(idx, inc, pr)
        assert all(np.array_equal(x, y) for x, y in zip(a, b))
        ga = oracle.snn_graph_shared(idx, inc, pr)
        gb = ref_oracle.snn_graph_shared(idx, inc, pr)
        assert all(np.array_equal(x, y) for x, y in zip(ga, gb))
