"""Python mirror of sparseDist's R interface for the blocked kNN path.

``sparseKNN``, ``sparseKNNCross``, ``sparseSNN`` and the two-matrix
``sparseDist`` keep the reference's argument names, defaults, validation
order and error text (R/sparseKNN.R, R/sparseKNNCross.R, R/sparseSNN.R,
R/sparseDist.R, R/utils-validate.R); the computation is libsdgpu.so on the
GPU.  R objects map onto Python ones as follows:

* a dgCMatrix (observations in the columns) -> a ``scipy.sparse`` matrix;
  dense numpy arrays are coerced the way ``.as_csparse`` coerces them;
* an ``ncol x k`` integer / double matrix -> a numpy array of shape (ncol, k)
  with R's NA encodings: ``NA_INTEGER`` (INT32_MIN) and ``NA_REAL`` (NaN with
  payload 1954); ``is_na()`` tests for either;
* ``attr(res, "self_search")`` -> ``KNNResult.self_search``;
* ``warning()`` -> ``warnings.warn`` (category ``SparseDistWarning``);
  ``stop()`` -> ``ValueError`` for argument errors, ``SdgError`` for failures
  reported by the library (which carry the reference's message text).
"""
from __future__ import annotations

import math
import numbers
import os
import sys
import warnings

import numpy as np

from . import _lib
from ._lib import NA_INTEGER, NA_REAL_BITS, SdgError

INT_MAX = 2 ** 31 - 1
METHOD_CHOICES = ("binary", "jaccard", "cosine", "euclidean", "manhattan", "pearson", "js",
                  "covariance")
METHOD_CODES = {"binary": 0, "cosine": 1, "euclidean": 2, "manhattan": 3, "pearson": 4, "js": 5,
                "covariance": 6}
NA_REAL = np.array([NA_REAL_BITS], dtype=np.uint64).view(np.float64)[0]


class SparseDistWarning(UserWarning):
    pass


class KNNResult(dict):
    """``list(idx, dist)`` with ``attr(, "self_search")`` and row names."""

    def __init__(self, idx, dist, self_search, rownames=None):
        super().__init__(idx=idx, dist=dist)
        self.self_search = self_search
        self.rownames = rownames

    @property
    def idx(self):
        return self["idx"]

    @property
    def dist(self):
        return self["dist"]


def is_na(a) -> np.ndarray:
    """R's is.na() for the arrays this module returns."""
    a = np.asarray(a)
    if a.dtype.kind == "f":
        return np.isnan(a)
    return a == NA_INTEGER


# ---------------------------------------------------------------------------
# validators: R/utils-validate.R:17-42 (and the local copies in sparseKNN())
# ---------------------------------------------------------------------------
def _is_bool_scalar(v):
    return isinstance(v, (bool, np.bool_))


def _chk_flag(value, name):
    if not _is_bool_scalar(value):
        raise ValueError("'%s' must be TRUE or FALSE." % name)


def _chk_count(value, name, allow_zero=False):
    lower = 0 if allow_zero else 1
    if isinstance(value, np.ndarray) and value.shape == ():
        value = value[()]
    ok = isinstance(value, numbers.Real) and not _is_bool_scalar(value)
    if ok:
        v = float(value)
        ok = math.isfinite(v) and v == math.floor(v) and v >= lower and v <= INT_MAX
    if not ok:
        raise ValueError("'%s' must be a %s integer no larger than .Machine$integer.max."
                         % (name, "non-negative" if allow_zero else "positive"))
    return int(value)


def _match_arg(arg, choices):
    """R's match.arg(): exact, then unique partial matching; a vector equal
    to the choices selects the first."""
    if isinstance(arg, (tuple, list)):
        if tuple(arg) == tuple(choices):
            return choices[0]
        if len(arg) != 1:
            raise ValueError("'arg' must be of length 1")
        arg = arg[0]
    if not isinstance(arg, str):
        raise ValueError("'arg' must be NULL or a character vector")
    if arg in choices:
        return arg
    hits = [c for c in choices if c.startswith(arg)] if arg else []
    if len(hits) == 1:
        return hits[0]
    raise ValueError("'arg' should be one of " + ", ".join("‘%s’" % c for c in choices))


def _detect_cores():
    """.detect_cores(): all cores minus one, at least 1 (R/sparseDist.R:221-224)."""
    n = os.cpu_count() or 1
    return 1 if n < 2 else n - 1


def _as_csparse(M):
    """.as_csparse (R/sparseDist.R:198-202): sparse input is kept as is
    (explicit zeros included); dense input drops its zeros."""
    import scipy.sparse as sp
    if sp.issparse(M):
        M = sp.csc_matrix(M, dtype=np.float64)
        if not M.has_sorted_indices:
            M = M.sorted_indices()
        return M
    A = np.asarray(M, dtype=np.float64)
    if A.ndim != 2:
        raise ValueError("a matrix is required")
    return sp.csc_matrix(A)


def _held(M):
    return _lib.HeldCSC(M.shape[0], M.shape[1], M.indptr, M.indices, M.data)


def _colnames(M):
    return getattr(M, "colnames", None)


def _ncol(M):
    shape = getattr(M, "shape", None)
    if shape is None or len(shape) != 2:
        return None
    return int(shape[1])


def _progress(verbose):
    if verbose:
        sys.stdout.write("  |" + "=" * 70 + "| 100%\n")
        sys.stdout.flush()


def _unpack(buf, n, k):
    """Column-major n x k buffer -> (n, k) array."""
    return buf[: n * k].reshape(k, n).T


def _ctx(ctx):
    return ctx if ctx is not None else _lib.default_context()


# ---------------------------------------------------------------------------
# sparseKNN: R/sparseKNN.R:110-313
# ---------------------------------------------------------------------------
def sparseKNN(X, Y=None, k=10, method="binary", dist=True, include_self=False,
              drop_degenerate=True, block_size=256, ncores=1, verbose=True, *, ctx=None):
    if X is None:
        raise ValueError("'X' must be provided.")
    _chk_flag(dist, "dist")
    _chk_flag(include_self, "include_self")
    _chk_flag(drop_degenerate, "drop_degenerate")
    _chk_flag(verbose, "verbose")
    ncores = _chk_count(ncores, "ncores", allow_zero=True)
    k = _chk_count(k, "k")
    block_size = _chk_count(block_size, "block_size")
    if ncores == 0:
        ncores = _detect_cores()
    method = _match_arg(method, METHOD_CHOICES)
    if method == "jaccard":
        method = "binary"
    if method in ("euclidean", "manhattan", "js") and not dist:
        raise ValueError("'dist = FALSE' is only meaningful for methods \"binary\", \"cosine\" "
                         "and \"pearson\"; %s has no similarity form." % method)
    nmX = _colnames(X)
    nq = _ncol(X)
    if nq is None or nq < 1:
        raise ValueError("'X' must have at least one column.")
    selfmode = Y is None
    if not selfmode and X.shape[0] != Y.shape[0]:
        raise ValueError("'X' and 'Y' must have the same number of rows.")
    Xs = _held(_as_csparse(X))
    Ys = None if selfmode else _held(_as_csparse(Y))
    c = _ctx(ctx)
    idx = np.empty(nq * k, np.int32)
    dst = np.empty(nq * k, np.float64)
    keff = np.zeros(1, np.int32)
    flags = np.zeros(1, np.int32)
    st = c.lib.sdg_knn(c.handle, Xs.ref, None if selfmode else Ys.ref, METHOD_CODES[method],
                       int(bool(dist)), k, int(bool(include_self)), int(bool(drop_degenerate)),
                       block_size, ncores, idx.ctypes.data, dst.ctypes.data, keff.ctypes.data,
                       flags.ctypes.data)
    _lib.check(st)
    ke = int(keff[0])
    if flags[0] & _lib.WARN_CLAMP_FWD:
        warnings.warn("k (%d) exceeds the %d available neighbours; returning %d." % (k, ke, ke),
                      SparseDistWarning, stacklevel=2)
    _progress(verbose)
    return KNNResult(_unpack(idx, nq, ke), _unpack(dst, nq, ke), selfmode, nmX)


# ---------------------------------------------------------------------------
# sparseKNNCross: R/sparseKNNCross.R:44-199
# ---------------------------------------------------------------------------
def sparseKNNCross(X, Y=None, k=10, method=METHOD_CHOICES, dist=True, drop_degenerate=True,
                   block_size=256, ncores=1, verbose=True, *, ctx=None):
    if Y is None:
        raise ValueError("'Y' is required. For a single matrix use sparseKNN(), which already "
                         "exploits symmetry via the full/diag arguments.")
    _chk_flag(dist, "dist")
    _chk_flag(drop_degenerate, "drop_degenerate")
    _chk_flag(verbose, "verbose")
    ncores = _chk_count(ncores, "ncores", allow_zero=True)
    k = _chk_count(k, "k")
    block_size = _chk_count(block_size, "block_size")
    if ncores == 0:
        ncores = _detect_cores()
    method = _match_arg(method, METHOD_CHOICES)
    if method == "jaccard":
        method = "binary"
    if method in ("euclidean", "manhattan", "js") and not dist:
        raise ValueError("'dist = FALSE' is only meaningful for methods \"binary\", \"cosine\" "
                         "and \"pearson\"; %s has no similarity form." % method)
    if X.shape[0] != Y.shape[0]:
        raise ValueError("'X' and 'Y' must have the same number of rows.")
    nq, nr = _ncol(X), _ncol(Y)
    if nq is None or nq < 1:
        raise ValueError("'X' must have at least one column.")
    if nr is None or nr < 1:
        raise ValueError("'Y' must have at least one column.")
    nmX, nmY = _colnames(X), _colnames(Y)
    Xs, Ys = _held(_as_csparse(X)), _held(_as_csparse(Y))
    c = _ctx(ctx)
    fi = np.empty(nq * k, np.int32); fd = np.empty(nq * k, np.float64)
    ri = np.empty(nr * k, np.int32); rd = np.empty(nr * k, np.float64)
    kf = np.zeros(1, np.int32); kr = np.zeros(1, np.int32); flags = np.zeros(1, np.int32)
    st = c.lib.sdg_knn_cross(c.handle, Xs.ref, Ys.ref, METHOD_CODES[method], int(bool(dist)), k,
                             int(bool(drop_degenerate)), block_size, ncores, fi.ctypes.data,
                             fd.ctypes.data, ri.ctypes.data, rd.ctypes.data, kf.ctypes.data,
                             kr.ctypes.data, flags.ctypes.data)
    _lib.check(st)
    f, r = int(kf[0]), int(kr[0])
    for bit, side, ke in ((_lib.WARN_CLAMP_FWD, "forward", f), (_lib.WARN_CLAMP_REV, "reverse", r)):
        if flags[0] & bit:
            warnings.warn("k (%d) exceeds the %d available neighbours for the %s direction; "
                          "returning %d." % (k, ke, side, ke), SparseDistWarning, stacklevel=2)
    _progress(verbose)
    return {"forward": KNNResult(_unpack(fi, nq, f), _unpack(fd, nq, f), False, nmX),
            "reverse": KNNResult(_unpack(ri, nr, r), _unpack(rd, nr, r), False, nmY)}


# ---------------------------------------------------------------------------
# sparseSNN: R/sparseSNN.R:120-251
# ---------------------------------------------------------------------------
def _idx_matrix(idx):
    if isinstance(idx, dict):
        ss = getattr(idx, "self_search", None)
        if ss is False:
            raise ValueError("sparseSNN() requires a self-search sparseKNN() result; the indices "
                             "from sparseKNN(X, Y) refer to the columns of Y, which are a "
                             "different node set.")
        if ss is not True:
            raise ValueError("'idx' must be a matrix, or a list produced by sparseKNN(). This "
                             "list carries no 'self_search' marker -- it may have been dropped by "
                             "subsetting -- so it cannot be confirmed to describe a single node "
                             "set. Pass the index matrix itself if that is intended.")
        if idx.get("idx") is None:
            raise ValueError("'idx' must be a matrix or the list returned by sparseKNN().")
        rown = getattr(idx, "rownames", None)
        idx = idx["idx"]
    else:
        rown = getattr(idx, "rownames", None)
    if not isinstance(idx, np.ndarray) or idx.ndim != 2:
        raise ValueError("'idx' must be a matrix or a sparseKNN() result.")
    n, k = idx.shape
    if n < 1 or k < 1:
        raise ValueError("'idx' must have at least one row and one column.")
    if idx.dtype.kind not in "iuf":
        raise ValueError("'idx' must be a numeric or integer matrix.")
    if idx.dtype.kind == "f":
        na = np.isnan(idx)
        v = np.where(na, 1.0, idx)
        bad = ~na & (~np.isfinite(v) | (v != np.floor(v)) | (v < 1) | (v > n))
        out = np.where(na, NA_INTEGER, np.where(bad, 0, v)).astype(np.int32)
    else:
        v = idx.astype(np.int64)
        na = v == NA_INTEGER
        bad = ~na & ((v < 1) | (v > n))
        out = v.astype(np.int32)
    if bad.any():
        raise ValueError("'idx' entries must be NA or finite, whole-number, 1-based row indices "
                         "in [1, nrow(idx)].")
    return np.asfortranarray(out), rown


def sparseSNN(idx, include_self=True, prune=0, symmetrise=None, edges=("knn", "shared"),
              ncores=1, verbose=True, *, ctx=None):
    import scipy.sparse as sp
    symmetrise_missing = symmetrise is None
    if symmetrise_missing:
        symmetrise = True
    M, rown = _idx_matrix(idx)
    n, k = M.shape
    _chk_flag(include_self, "include_self")
    _chk_flag(symmetrise, "symmetrise")
    _chk_flag(verbose, "verbose")
    edges = _match_arg(edges, ("knn", "shared"))
    if edges == "shared" and not symmetrise_missing and not symmetrise:
        warnings.warn("'symmetrise' is ignored when edges = \"shared\": that edge set is "
                      "symmetric by construction.", SparseDistWarning, stacklevel=2)
    if (not isinstance(prune, numbers.Real) or _is_bool_scalar(prune) or
            not math.isfinite(float(prune)) or prune < 0 or prune > 1):
        raise ValueError("'prune' must be a finite number between 0 and 1.")
    if (not isinstance(ncores, numbers.Real) or _is_bool_scalar(ncores) or
            not math.isfinite(float(ncores)) or ncores != math.floor(ncores) or ncores < 0 or
            ncores > INT_MAX):
        raise ValueError("'ncores' must be a non-negative integer no larger than "
                         ".Machine$integer.max.")
    c = _ctx(ctx)
    nnz = np.zeros(1, np.int64)
    if edges == "shared":
        # snnJaccardShared + sparseMatrix(symmetric = TRUE) (R/sparseSNN.R:202-219)
        def call(p_, i_, x_):
            _lib.check(c.lib.sdg_snn_graph_shared(c.handle, M.ctypes.data, n, k, int(bool(include_self)),
                                                  float(prune), nnz.ctypes.data, p_, i_, x_))
    else:
        def call(p_, i_, x_):
            _lib.check(c.lib.sdg_snn_graph(c.handle, M.ctypes.data, n, k, int(bool(include_self)),
                                           float(prune), int(bool(symmetrise)), nnz.ctypes.data,
                                           p_, i_, x_))
    call(None, None, None)
    m = int(nnz[0])
    p = np.empty(n + 1, np.int32)
    i = np.empty(max(m, 1), np.int32)
    x = np.empty(max(m, 1), np.float64)
    call(p.ctypes.data, i.ctypes.data, x.ctypes.data)
    _progress(verbose)
    g = sp.csc_matrix((x[:m], i[:m], p), shape=(n, n))
    g.rownames = rown
    return g


# ---------------------------------------------------------------------------
# sparseDist, two-matrix form: R/sparseDist.R:172-182
# ---------------------------------------------------------------------------
def sparseDist(X, Y=None, method="binary", ncores=1, verbose=True, full=False, diag=False,
               dist=True, *, ctx=None):
    """R/sparseDist.R:133-190.  With Y, the cross matrix D[i, j] = method(column
    i of X, column j of Y); without, the matrix among the columns of X: its
    lower triangle (full = False) or both (full = True), the diagonal as the
    reference's single-matrix kernels leave it (`diag` only decides whether
    the euclidean / manhattan / covariance self pairs are computed).

    Storage follows the reference's (src/sparseDist.cpp, RESULT STORAGE):
    distance-valued results are a dense ndarray; coefficient-valued ones
    (covariance, and binary / cosine / pearson with dist = False) a
    scipy.sparse.csc_matrix holding the non-zero entries."""
    if X is None:
        raise ValueError("'X' must be provided.")
    method = _match_arg(method, METHOD_CHOICES)
    if method == "jaccard":
        method = "binary"
    c = _ctx(ctx)
    Xs = _held(_as_csparse(X))
    if Y is None:
        n = Xs.ncol
        D = np.empty((n, n), np.float64)
        _lib.check(c.lib.sdg_dist(c.handle, METHOD_CODES[method], int(bool(dist)), Xs.ref,
                                  int(bool(full)), int(bool(diag)), D.ctypes.data))
    else:
        Ys = _held(_as_csparse(Y))
        D = np.empty((Ys.ncol, Xs.ncol), np.float64)
        _lib.check(c.lib.sdg_dist_cross(c.handle, METHOD_CODES[method], int(bool(dist)), Xs.ref,
                                        Ys.ref, D.ctypes.data))
    D = D.T
    if method == "covariance" or (method in ("binary", "cosine", "pearson") and not dist):
        import scipy.sparse as sp
        return sp.csc_matrix(D)
    return D


# ---------------------------------------------------------------------------
# the reference's internal kernels (sparseDist:::topKBlock and friends)
# ---------------------------------------------------------------------------
def topKBlock(D, k, decreasing, self_row, ncores=1, *, ctx=None):
    """src/topK.cpp:66-149 -> {'idx': (ncol, k) int32, 'dist': (ncol, k) float64}."""
    D = np.asfortranarray(D, dtype=np.float64)
    nrow, ncol = D.shape
    sr = np.atleast_1d(np.asarray(self_row))
    if sr.size != ncol:
        raise ValueError("self_row must have one entry per column of D.")
    sr = np.ascontiguousarray(sr, dtype=np.int32)
    k = int(k)
    c = _ctx(ctx)
    kk = max(k, 1)
    idx = np.empty(ncol * kk, np.int32)
    dst = np.empty(ncol * kk, np.float64)
    _lib.check(c.lib.sdg_topk_block(c.handle, D.ctypes.data, nrow, ncol, k, int(bool(decreasing)),
                                    sr.ctypes.data, idx.ctypes.data, dst.ctypes.data))
    return {"idx": _unpack(idx, ncol, k), "dist": _unpack(dst, ncol, k)}


def topKRowsAccum(D, k, decreasing, best_idx, best_val, col_offset, self_col, ncores=1,
                  tile_rows=64, *, ctx=None):
    """src/topKRows.cpp:103-248: updates best_idx / best_val (Fortran-ordered
    (nrow, k) arrays) in place, as the reference mutates its R matrices."""
    D = np.asfortranarray(D, dtype=np.float64)
    nrow, ncol = D.shape
    k = int(k)
    if (best_idx.shape != (nrow, k) or best_val.shape != (nrow, k) or
            not best_idx.flags.f_contiguous or not best_val.flags.f_contiguous or
            best_idx.dtype != np.int32 or best_val.dtype != np.float64):
        raise ValueError("best_idx and best_val must both be nrow(D) x k.")
    sc = np.ascontiguousarray(self_col, dtype=np.int32)
    if sc.size != nrow:
        raise ValueError("self_col must have one entry per row of D.")
    c = _ctx(ctx)
    _lib.check(c.lib.sdg_topk_rows_accum(c.handle, D.ctypes.data, nrow, ncol, k,
                                         int(bool(decreasing)), best_idx.ctypes.data,
                                         best_val.ctypes.data, int(col_offset), sc.ctypes.data))


def snnJaccard(idx, include_self=True, ncores=1, verbose=False, *, ctx=None):
    """src/snn.cpp:197-250 -> (n, k) float64 weights aligned with idx."""
    M = np.asfortranarray(idx, dtype=np.int32)
    n, k = M.shape
    c = _ctx(ctx)
    w = np.empty(max(n * k, 1), np.float64)
    _lib.check(c.lib.sdg_snn_jaccard(c.handle, M.ctypes.data, n, k, int(bool(include_self)),
                                     w.ctypes.data))
    return _unpack(w, n, k)
