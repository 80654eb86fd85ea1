"""ctypes bindings for the CPU oracle (test infrastructure only).

``Oracle()`` wraps ``oracle/_build/libsdgoracle.so`` (the C restatement) and
``Oracle(ref=True)`` wraps ``oracle/_ref/libsdref.so`` (the reference's own
kernels compiled against the shim).  Both expose the same calls, taking
scipy CSC matrices and returning numpy arrays laid out like the R results
(column-major n x k matrices are returned as numpy arrays of shape (n, k)).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs use
this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

NA_INT = np.int32(-(2 ** 31))
NA_REAL_BITS = np.uint64(0x7FF00000000007A2)

METHODS = {"binary": 0, "jaccard": 0, "cosine": 1, "euclidean": 2, "manhattan": 3,
           "pearson": 4, "js": 5, "covariance": 6}


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class _CSC(C.Structure):
    _fields_ = [("nrow", C.c_int32), ("ncol", C.c_int32),
                ("p", C.POINTER(C.c_int32)), ("i", C.POINTER(C.c_int32)),
                ("x", C.POINTER(C.c_double))]


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def as_csc_arrays(M):
    """(nrow, ncol, p int32, i int32, x float64) of a scipy sparse matrix."""
    import scipy.sparse as sp
    M = sp.csc_matrix(M)
    if not M.has_sorted_indices:
        M = M.sorted_indices()
    return (int(M.shape[0]), int(M.shape[1]), np.ascontiguousarray(M.indptr, np.int32),
            np.ascontiguousarray(M.indices, np.int32), np.ascontiguousarray(M.data, np.float64))


class _Held:
    """Keeps the numpy buffers alive for the lifetime of the ctypes struct."""

    def __init__(self, M):
        self.nrow, self.ncol, self.p, self.i, self.x = as_csc_arrays(M)
        self.s = _CSC(self.nrow, self.ncol, _ptr(self.p, C.c_int32), _ptr(self.i, C.c_int32),
                      _ptr(self.x, C.c_double))


def na_real_array(shape):
    return np.full(shape, NA_REAL_BITS, dtype=np.uint64).view(np.float64)


class Oracle:
    def __init__(self, ref: bool = False, threads: int = 1):
        self.ref = ref
        if ref:
            path = _build.build_ref()
            if path is None:
                path = _build.REF_SO
            if not os.path.exists(path):
                raise FileNotFoundError("reference build unavailable: " + path)
            self.lib = C.CDLL(path)
            pre = "ref_"
            self.lib.ref_last_error.restype = C.c_char_p
            self._err = self.lib.ref_last_error
            self.lib.ref_set_threads(int(threads))
        else:
            self.lib = C.CDLL(_build.build_oracle())
            pre = "orc_"
            self.lib.orc_last_error.restype = C.c_char_p
            self._err = self.lib.orc_last_error
            self.lib.orc_set_threads(int(threads))
        self._slab = getattr(self.lib, pre + ("slab_c" if ref else "slab"))
        self._dist = getattr(self.lib, pre + ("dist_c" if ref else "dist"))
        self._dist.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        self._topk = getattr(self.lib, pre + ("topk_block_c" if ref else "topk_block"))
        self._rows = getattr(self.lib, pre + ("topk_rows_accum_c" if ref else "topk_rows_accum"))
        self._snn = getattr(self.lib, pre + ("snn_jaccard_c" if ref else "snn_jaccard"))
        self._knn = getattr(self.lib, pre + "knn")
        self._cross = getattr(self.lib, pre + "knn_cross")
        self._graph = getattr(self.lib, pre + "snn_graph")
        self._shared = getattr(self.lib, pre + ("snn_shared_c" if ref else "snn_shared"))
        self._graph_shared = getattr(self.lib, pre + "snn_graph_shared")
        self._shared.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int, C.c_double, C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_void_p]
        self._graph_shared.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int, C.c_double,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        for f in (self._topk, self._rows):
            f.argtypes = None
        self._topk.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int, C.c_int,
                               C.c_void_p, C.c_void_p, C.c_void_p]
        self._rows.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int, C.c_int,
                               C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
        self._snn.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int, C.c_void_p]
        self._graph.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int, C.c_double, C.c_int,
                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]

    def set_threads(self, n: int):
        (self.lib.ref_set_threads if self.ref else self.lib.orc_set_threads)(int(n))

    def _check(self, st):
        if st != 0:
            raise OracleError(st, self._err().decode())

    # -- kernels ---------------------------------------------------------------
    def slab(self, method, m, m2, dist=True):
        a, b = _Held(m), _Held(m2)
        D = np.zeros((b.ncol, a.ncol), dtype=np.float64)     # column-major nc x nc2
        self._check(self._slab(METHODS[method], int(dist), C.byref(a.s), C.byref(b.s),
                               _ptr(D, C.c_double)))
        return D.T

    def dist_single(self, method, m, full=False, diag=False, dist=True):
        """Single-matrix sparseDist(X): the dense n x n accumulator of the
        reference's fastJacc / fastCosine / ... / fastCov (before the R-level
        dense-or-sparse storage choice)."""
        a = _Held(m)
        D = np.zeros((a.ncol, a.ncol), dtype=np.float64)     # column-major n x n
        self._check(self._dist(METHODS[method], int(dist), C.byref(a.s), int(bool(full)),
                               int(bool(diag)), _ptr(D, C.c_double)))
        return D.T

    def topk_block(self, D, k, decreasing, self_row):
        D = np.asfortranarray(D, dtype=np.float64)
        nrow, ncol = D.shape
        sr = np.ascontiguousarray(self_row, dtype=np.int32)
        idx = np.empty((k, ncol), np.int32)
        dst = np.empty((k, ncol), np.float64)
        self._check(self._topk(D.ctypes.data, nrow, ncol, int(k), int(decreasing),
                               sr.ctypes.data, idx.ctypes.data, dst.ctypes.data))
        return idx.T.copy(), dst.T.copy()

    def topk_rows_accum(self, D, k, decreasing, best_idx, best_val, col_offset, self_col):
        D = np.asfortranarray(D, dtype=np.float64)
        nrow, ncol = D.shape
        bi = np.asfortranarray(best_idx, dtype=np.int32)
        bv = np.asfortranarray(best_val, dtype=np.float64)
        sc = np.ascontiguousarray(self_col, dtype=np.int32)
        self._check(self._rows(D.ctypes.data, nrow, ncol, int(k), int(decreasing),
                               bi.ctypes.data, bv.ctypes.data, int(col_offset), sc.ctypes.data))
        return bi, bv

    def snn_jaccard(self, idx, include_self=True):
        idx = np.asfortranarray(idx, dtype=np.int32)
        n, k = idx.shape
        w = np.empty((k, n), np.float64)
        self._check(self._snn(idx.ctypes.data, n, k, int(include_self), w.ctypes.data))
        return w.T.copy()

    # -- orchestration -----------------------------------------------------------
    def knn(self, X, Y=None, k=10, method="binary", dist=True, include_self=False,
            drop_degenerate=True, block_size=256):
        a = _Held(X)
        b = _Held(Y) if Y is not None else None
        nq = a.ncol
        idx = np.empty(nq * k, np.int32)
        dst = np.empty(nq * k, np.float64)
        keff = C.c_int(0)
        flags = C.c_int(0)
        st = self._knn(C.byref(a.s), C.byref(b.s) if b else None, METHODS[method], int(dist),
                       int(k), int(include_self), int(drop_degenerate), int(block_size),
                       _ptr(idx, C.c_int32), _ptr(dst, C.c_double), C.byref(keff),
                       C.byref(flags))
        self._check(st)
        ke = keff.value
        return (idx[:nq * ke].reshape(ke, nq).T.copy(), dst[:nq * ke].reshape(ke, nq).T.copy(),
                flags.value)

    def knn_cross(self, X, Y, k=10, method="binary", dist=True, drop_degenerate=True,
                  block_size=256):
        a, b = _Held(X), _Held(Y)
        nq, nr = a.ncol, b.ncol
        fi = np.empty(nq * k, np.int32); fd = np.empty(nq * k, np.float64)
        ri = np.empty(nr * k, np.int32); rd = np.empty(nr * k, np.float64)
        kf, kr, flags = C.c_int(0), C.c_int(0), C.c_int(0)
        st = self._cross(C.byref(a.s), C.byref(b.s), METHODS[method], int(dist), int(k),
                         int(drop_degenerate), int(block_size), _ptr(fi, C.c_int32),
                         _ptr(fd, C.c_double), _ptr(ri, C.c_int32), _ptr(rd, C.c_double),
                         C.byref(kf), C.byref(kr), C.byref(flags))
        self._check(st)
        f, r = kf.value, kr.value
        return ((fi[:nq * f].reshape(f, nq).T.copy(), fd[:nq * f].reshape(f, nq).T.copy()),
                (ri[:nr * r].reshape(r, nr).T.copy(), rd[:nr * r].reshape(r, nr).T.copy()),
                flags.value)

    def snn_shared(self, idx, include_self=True, prune=0.0):
        """snnJaccardShared: (i, j, x) upper-triangle triplets, 1-based, in the
        kernel's order."""
        idx = np.asfortranarray(idx, dtype=np.int32)
        n, k = idx.shape
        m = C.c_int64(0)
        self._check(self._shared(idx.ctypes.data, n, k, int(include_self), float(prune),
                                 C.addressof(m), None, None, None))
        ti = np.empty(max(m.value, 1), np.int32)
        tj = np.empty(max(m.value, 1), np.int32)
        tx = np.empty(max(m.value, 1), np.float64)
        self._check(self._shared(idx.ctypes.data, n, k, int(include_self), float(prune),
                                 C.addressof(m), ti.ctypes.data, tj.ctypes.data, tx.ctypes.data))
        return ti[:m.value], tj[:m.value], tx[:m.value]

    def snn_graph_shared(self, idx, include_self=True, prune=0.0):
        """Returns (p, i, x) of the symmetric n x n dgCMatrix of edges = "shared"."""
        idx = np.asfortranarray(idx, dtype=np.int32)
        n, k = idx.shape
        nnz = C.c_int64(0)
        self._check(self._graph_shared(idx.ctypes.data, n, k, int(include_self), float(prune),
                                       C.addressof(nnz), None, None, None))
        p = np.empty(n + 1, np.int32)
        i = np.empty(max(nnz.value, 1), np.int32)
        x = np.empty(max(nnz.value, 1), np.float64)
        self._check(self._graph_shared(idx.ctypes.data, n, k, int(include_self), float(prune),
                                       C.addressof(nnz), p.ctypes.data, i.ctypes.data,
                                       x.ctypes.data))
        return p, i[:nnz.value], x[:nnz.value]

    def snn_graph(self, idx, include_self=True, prune=0.0, symmetrise=True):
        """Returns (p, i, x) of the n x n dgCMatrix."""
        idx = np.asfortranarray(idx, dtype=np.int32)
        n, k = idx.shape
        nnz = C.c_int64(0)
        self._check(self._graph(idx.ctypes.data, n, k, int(include_self), float(prune),
                                int(symmetrise), C.addressof(nnz), None, None, None))
        p = np.empty(n + 1, np.int32)
        i = np.empty(max(nnz.value, 1), np.int32)
        x = np.empty(max(nnz.value, 1), np.float64)
        self._check(self._graph(idx.ctypes.data, n, k, int(include_self), float(prune),
                                int(symmetrise), C.addressof(nnz), p.ctypes.data, i.ctypes.data,
                                x.ctypes.data))
        return p, i[:nnz.value], x[:nnz.value]
