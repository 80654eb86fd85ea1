"""Pins the CPU oracle before the GPU results are compared with it:

* against the committed outputs of the reference's own kernels
  (tests/golden, made by tests/golden/make_golden.py from oracle/_ref);
* against the literal fixtures / known answers of the reference's testthat
  suite (parity_cases.KNOWN_ANSWERS);
* against oracle/_ref directly on randomised inputs, where the reference
  checkout is present (bit for bit for the pinned methods).
"""
import numpy as np
import pytest

from backends import OracleBackend, load_golden, make_x, normalise_cols, same_bits
from parity_cases import KNOWN_ANSWERS, check_golden_case

CASES, ARR = load_golden()


@pytest.fixture(scope="module")
def orc():
    return OracleBackend()


@pytest.mark.parametrize("case", CASES, ids=[c["id"] for c in CASES])
def test_oracle_matches_reference_golden(orc, case):
    check_golden_case(orc, case, ARR)


@pytest.mark.parametrize("fn", KNOWN_ANSWERS, ids=[f.__name__ for f in KNOWN_ANSWERS])
def test_oracle_known_answers(orc, fn):
    fn(orc)


@pytest.mark.parametrize("method", ["binary", "cosine", "euclidean", "manhattan", "pearson", "js",
                                    "covariance"])
def test_oracle_bit_identical_to_reference_build(ref_oracle, method):
    orc = OracleBackend()
    rng = np.random.default_rng(7)
    for trial in range(6):
        n = int(rng.integers(30, 120))
        X = make_x(n, int(rng.integers(2, 30)), float(rng.uniform(0.03, 0.3)), 100 + trial)
        Y = make_x(n, int(rng.integers(2, 30)), float(rng.uniform(0.03, 0.3)), 200 + trial)
        if method == "js":
            X, Y = normalise_cols(X), normalise_cols(Y)
        a = orc.slab(method, X, Y, True)
        b = ref_oracle.slab(method, X, Y, True)
        assert same_bits(np.ascontiguousarray(a), np.ascontiguousarray(b))
        k = int(rng.integers(1, 8))
        a = orc.knn_cross(X, Y, k=k, method=method, block_size=int(rng.integers(1, 9)))
        b = ref_oracle.knn_cross(X, Y, k=k, method=method, block_size=int(rng.integers(1, 9)))
        for u, v in zip(a[0] + a[1], b[0] + b[1]):
            assert same_bits(u, v)
