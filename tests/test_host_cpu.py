"""Host-side checks that need no GPU: the C ABI library loads and exports
every symbol include/sdgpu.h declares, and the Python mirror of the R API
validates its arguments with the reference's messages, in the reference's
order, before anything reaches the device."""
import os
import re

import numpy as np
import pytest
import scipy.sparse as sp

import sparsedist_gb300 as sdg
from backends import make_x

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "sdgpu.h")).read()
    return sorted(set(re.findall(r"SDG_API\s+[\w\s\*]+?\b(sdg_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    syms = declared_symbols()
    assert len(syms) >= 15
    lib = sdg.load_library()
    missing = [s for s in syms if not hasattr(lib, s)]
    assert missing == []
    assert lib.sdg_version() >= 10000


def test_error_buffer_roundtrip():
    from sparsedist_gb300 import _lib
    lib = _lib.load()
    # an argument error raised before any device work
    st = lib.sdg_ctx_set_engine(None, 0)
    assert st == -1
    assert "engine" in _lib.last_error()


X = make_x(60, 12, 0.3, 1)


@pytest.mark.parametrize("kw,msg", [
    (dict(k=0), "'k' must be a positive integer"),
    (dict(k=-1), "'k' must be a positive integer"),
    (dict(block_size=0), "'block_size' must be a positive integer"),
    (dict(k=2.5), "positive integer"),
    (dict(block_size=4.5), "positive integer"),
    (dict(k=3, ncores=1.7), "non-negative integer"),
    (dict(k=3, ncores=float("inf")), "non-negative integer"),
    (dict(k=float("inf")), "positive integer"),
    (dict(k=[2, 3]), "positive integer"),
    (dict(k="3"), "positive integer"),
    (dict(k=3e9), "integer.max"),
    (dict(k=3, block_size=3e9), "integer.max"),
    (dict(k=3, ncores=3e9), "integer.max"),
    (dict(k=True), "positive integer"),
])
def test_count_validation(kw, msg):
    # test-sparseKNN.R:123-143, :314-324
    with pytest.raises(ValueError, match=re.escape(msg)):
        sdg.sparseKNN(X, verbose=False, **kw)


@pytest.mark.parametrize("bad", [None, 1, "TRUE", (True, False), np.array([])])
def test_flag_validation(bad):
    # test-sparseKNN.R:242-252
    if bad is None:
        pytest.skip("None is R's NULL, handled as 'not provided'")
    with pytest.raises(ValueError, match="'dist' must be TRUE or FALSE"):
        sdg.sparseKNN(X, dist=bad, verbose=False)
    with pytest.raises(ValueError, match="'include_self' must be TRUE or FALSE"):
        sdg.sparseKNN(X, include_self=bad, verbose=False)


def test_distance_only_methods_reject_similarity():
    # test-sparseKNN.R:210-216
    for m in ("euclidean", "manhattan", "js"):
        with pytest.raises(ValueError, match="only meaningful"):
            sdg.sparseKNN(X, k=3, method=m, dist=False, verbose=False)


def test_method_matching():
    from sparsedist_gb300.api import _match_arg, METHOD_CHOICES
    assert _match_arg("cos", METHOD_CHOICES) == "cosine"
    assert _match_arg(METHOD_CHOICES, METHOD_CHOICES) == "binary"
    with pytest.raises(ValueError, match="should be one of"):
        _match_arg("nope", METHOD_CHOICES)
    # match.arg's partial matching: "cov" is covariance, "co" is ambiguous
    assert _match_arg("cov", METHOD_CHOICES) == "covariance"
    with pytest.raises(ValueError, match="should be one of"):
        _match_arg("co", METHOD_CHOICES)
    # sparseDist validates the method before it needs a device
    with pytest.raises(ValueError, match="should be one of"):
        sdg.sparseDist(make_x(20, 4, 0.3, 1), method="nope", verbose=False)
    with pytest.raises(ValueError, match="must be provided"):
        sdg.sparseDist(None, verbose=False)


def test_rows_and_columns_checked_first():
    # test-sparseKNN.R:232-237
    Z = make_x(50, 8, 0.3, 3)
    with pytest.raises(ValueError, match="same number of rows"):
        sdg.sparseKNN(make_x(60, 8, 0.3, 1), Z, k=3, verbose=False)
    with pytest.raises(ValueError, match="at least one column"):
        sdg.sparseKNN(sp.csc_matrix((5, 0)), k=1, verbose=False)


def test_cross_validation_messages():
    # test-sparseKNNCross.R:166-173, :198-241
    Xb = make_x(80, 12, 0.1, 41, binary=True)
    Yb = make_x(80, 9, 0.1, 42, binary=True)
    with pytest.raises(ValueError, match="required"):
        sdg.sparseKNNCross(Xb, verbose=False)
    with pytest.raises(ValueError, match="same number of rows"):
        sdg.sparseKNNCross(Xb, make_x(59, 10, 0.1, 14), k=3, verbose=False)
    for kw, msg in ((dict(k=2.5), "'k' must be a positive integer"),
                    (dict(k=0), "'k' must be a positive integer"),
                    (dict(block_size=4.5), "'block_size' must be a positive integer"),
                    (dict(ncores=-1), "'ncores' must be a non-negative integer"),
                    (dict(dist=1), "'dist' must be TRUE or FALSE"),
                    (dict(drop_degenerate=1), "'drop_degenerate' must be TRUE or FALSE"),
                    (dict(verbose=1), "'verbose' must be TRUE or FALSE")):
        with pytest.raises(ValueError, match=re.escape(msg)):
            sdg.sparseKNNCross(Xb, Yb, **({"verbose": False} | kw))


def test_snn_validation_messages():
    # test-sparseSNN.R:139-150, :192-216
    idx = np.array([[2, 3], [1, 3], [1, 2]], np.int32)
    with pytest.raises(ValueError, match="TRUE or FALSE"):
        sdg.sparseSNN(idx, include_self=np.nan, verbose=False)
    with pytest.raises(ValueError, match="TRUE or FALSE"):
        sdg.sparseSNN(idx, symmetrise=1, verbose=False)
    for bad in (-0.1, 1.5, float("inf"), float("nan")):
        with pytest.raises(ValueError, match="between 0 and 1"):
            sdg.sparseSNN(idx, prune=bad, verbose=False)
    with pytest.raises(ValueError, match="non-negative integer"):
        sdg.sparseSNN(idx, ncores=1.5, verbose=False)
    with pytest.raises(ValueError, match="sparseKNN"):
        sdg.sparseSNN({"a": 1}, verbose=False)
    with pytest.raises(ValueError, match="matrix"):
        sdg.sparseSNN("nope", verbose=False)
    with pytest.raises(ValueError, match="whole-number"):
        sdg.sparseSNN(np.full((1, 1), 1.5), verbose=False)
    with pytest.raises(ValueError, match="finite"):
        sdg.sparseSNN(np.full((1, 1), np.inf), verbose=False)
    with pytest.raises(ValueError, match="numeric or integer"):
        sdg.sparseSNN(np.full((1, 1), "1"), verbose=False)
    with pytest.raises(ValueError, match="1-based"):
        sdg.sparseSNN(np.zeros((1, 1), np.int32), verbose=False)
    cross = sdg.KNNResult(idx, idx.astype(float), False)
    with pytest.raises(ValueError, match="self-search"):
        sdg.sparseSNN(cross, verbose=False)
    stripped = {"idx": idx, "dist": idx.astype(float)}
    with pytest.raises(ValueError, match="self_search"):
        sdg.sparseSNN(stripped, verbose=False)
