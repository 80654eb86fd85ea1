"""Pins the oracle's single-matrix sparseDist(X) restatement: against the
known answers of the reference's test-sparseDist.R, and bit for bit against
the reference's own single-matrix kernels built into oracle/_ref (every
method, full / diag / dist, ragged sizes and degenerate columns)."""
import numpy as np
import pytest

from backends import OracleBackend, same_bits
from dist_cases import KNOWN_DIST, METHODS, random_dist_cases


@pytest.fixture(scope="module")
def orc():
    return OracleBackend()


@pytest.mark.parametrize("fn", KNOWN_DIST, ids=[f.__name__ for f in KNOWN_DIST])
def test_oracle_dist_known_answers(orc, fn):
    fn(orc)


def test_oracle_dist_bit_identical_to_reference_build(ref_oracle):
    orc = OracleBackend()
    n = 0
    for method, X, full, diag, dist in random_dist_cases(21, 3):
        a = orc.dist_single(method, X, full, diag, dist)
        b = ref_oracle.dist_single(method, X, full, diag, dist)
        assert same_bits(np.ascontiguousarray(a), np.ascontiguousarray(b)), (method, X.shape, full, diag, dist)
        n += 1
    assert n > 100


@pytest.mark.parametrize("method", METHODS)
def test_oracle_dist_lower_is_cross_upper(orc, method):
    """The single-matrix value of the pair i < j is the two-matrix kernel's
    value of (column i, column j): both reach the same pair arithmetic."""
    from dist_cases import make_p
    from backends import make_x
    X = make_p(70, 12, 0.3, 4) if method == "js" else make_x(70, 12, 0.3, 4)
    D = orc.dist_single(method, X, False, False, True)
    S = orc.slab(method, X, X, True)
    i, j = np.triu_indices(X.shape[1], 1)
    assert same_bits(np.ascontiguousarray(D[j, i]), np.ascontiguousarray(S[i, j]))
