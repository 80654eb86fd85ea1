"""Uniform test adapters over the three implementations of the path:
the CPU oracle (oracle/sdg_oracle.c), the reference's own kernels
(oracle/_ref) and the GPU library (libsdgpu.so through its C ABI).

Every adapter returns numpy arrays shaped like the R results ((n, k) for an
n x k matrix) plus the clamp-warning flags."""
from __future__ import annotations

import json
import os

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
METHODS = {"binary": 0, "jaccard": 0, "cosine": 1, "euclidean": 2, "manhattan": 3,
           "pearson": 4, "js": 5, "covariance": 6}
NA_INT = np.int32(-(2 ** 31))


def make_x(n, p, density, seed, binary=False, signed=False):
    """make_X() of the reference's tests (abs(rsparsematrix(n, p, density)))
    drawn with numpy: |N(0,1)| values on a uniform random pattern."""
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
    M = M.multiply(1.0 / s[keep][None, :]).tocsc()
    M.sort_indices()
    return M


def same_bits(a, b):
    """Bit-for-bit equality of two arrays (NaN payloads included)."""
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    if a.shape != b.shape or a.dtype != b.dtype:
        return False
    return np.array_equal(a.view(np.uint8), b.view(np.uint8))


def load_golden():
    with open(os.path.join(HERE, "golden", "golden.json")) as f:
        meta = json.load(f)
    arr = np.load(os.path.join(HERE, "golden", "golden.npz"))
    return meta["cases"], arr


def golden_matrix(arr, name):
    nrow, ncol = arr[name + "_dim"]
    return sp.csc_matrix((arr[name + "_x"], arr[name + "_i"], arr[name + "_p"]), shape=(nrow, ncol))


class OracleBackend:
    def __init__(self, ref=False):
        from oracle.pyoracle import Oracle
        self.o = Oracle(ref=ref)

    def knn(self, X, Y=None, **kw):
        return self.o.knn(X, Y, **kw)

    def knn_cross(self, X, Y, **kw):
        return self.o.knn_cross(X, Y, **kw)

    def slab(self, method, m, m2, dist=True):
        return self.o.slab(method, m, m2, dist)

    def dist_single(self, method, m, full=False, diag=False, dist=True):
        return self.o.dist_single(method, m, full, diag, dist)

    def topk_block(self, D, k, decreasing, self_row):
        return self.o.topk_block(D, k, decreasing, self_row)

    def topk_rows_accum(self, D, k, decreasing, best_idx, best_val, col_offset, self_col):
        return self.o.topk_rows_accum(D, k, decreasing, best_idx, best_val, col_offset, self_col)

    def snn_jaccard(self, idx, include_self=True):
        return self.o.snn_jaccard(idx, include_self)

    def snn_graph(self, idx, include_self=True, prune=0.0, symmetrise=True):
        return self.o.snn_graph(idx, include_self, prune, symmetrise)


class GpuBackend:
    """Calls libsdgpu.so's C ABI directly (ctypes), as an FFI binding would."""

    def __init__(self, engine=0):
        from sparsedist_gb300 import _lib
        self.L = _lib
        self.ctx = _lib.Context()
        self.ctx.set_engine(engine)
        self.lib = self.ctx.lib
        self.h = self.ctx.handle

    def set_engine(self, e):
        self.ctx.set_engine(e)

    def _held(self, M):
        M = sp.csc_matrix(M)
        M.sort_indices()
        return self.L.HeldCSC(M.shape[0], M.shape[1], M.indptr, M.indices, M.data)

    def knn(self, X, Y=None, k=10, method="binary", dist=True, include_self=False,
            drop_degenerate=True, block_size=256):
        a = self._held(X)
        b = self._held(Y) if Y is not None else None
        nq = a.ncol
        idx = np.empty(nq * k, np.int32)
        dst = np.empty(nq * k, np.float64)
        ke, fl = np.zeros(1, np.int32), np.zeros(1, np.int32)
        self.L.check(self.lib.sdg_knn(self.h, a.ref, b.ref if b else None, METHODS[method],
                                      int(dist), int(k), int(include_self), int(drop_degenerate),
                                      int(block_size), 1, idx.ctypes.data, dst.ctypes.data,
                                      ke.ctypes.data, fl.ctypes.data))
        e = int(ke[0])
        return (idx[:nq * e].reshape(e, nq).T.copy(), dst[:nq * e].reshape(e, nq).T.copy(),
                int(fl[0]))

    def knn_cross(self, X, Y, k=10, method="binary", dist=True, drop_degenerate=True,
                  block_size=256):
        a, b = self._held(X), self._held(Y)
        nq, nr = a.ncol, b.ncol
        fi = np.empty(nq * k, np.int32); fd = np.empty(nq * k, np.float64)
        ri = np.empty(nr * k, np.int32); rd = np.empty(nr * k, np.float64)
        kf, kr, fl = np.zeros(1, np.int32), np.zeros(1, np.int32), np.zeros(1, np.int32)
        self.L.check(self.lib.sdg_knn_cross(self.h, a.ref, b.ref, METHODS[method], int(dist),
                                            int(k), int(drop_degenerate), int(block_size), 1,
                                            fi.ctypes.data, fd.ctypes.data, ri.ctypes.data,
                                            rd.ctypes.data, kf.ctypes.data, kr.ctypes.data,
                                            fl.ctypes.data))
        f, r = int(kf[0]), int(kr[0])
        return ((fi[:nq * f].reshape(f, nq).T.copy(), fd[:nq * f].reshape(f, nq).T.copy()),
                (ri[:nr * r].reshape(r, nr).T.copy(), rd[:nr * r].reshape(r, nr).T.copy()),
                int(fl[0]))

    def slab(self, method, m, m2, dist=True):
        a, b = self._held(m), self._held(m2)
        D = np.empty((b.ncol, a.ncol), np.float64)
        self.L.check(self.lib.sdg_dist_cross(self.h, METHODS[method], int(dist), a.ref, b.ref,
                                             D.ctypes.data))
        return D.T

    def dist_single(self, method, m, full=False, diag=False, dist=True):
        a = self._held(m)
        D = np.empty((a.ncol, a.ncol), np.float64)
        self.L.check(self.lib.sdg_dist(self.h, METHODS[method], int(dist), a.ref, int(bool(full)),
                                       int(bool(diag)), D.ctypes.data))
        return D.T

    def topk_block(self, D, k, decreasing, self_row):
        D = np.asfortranarray(D, dtype=np.float64)
        nrow, ncol = D.shape
        sr = np.ascontiguousarray(self_row, dtype=np.int32)
        idx = np.empty(max(ncol * k, 1), np.int32)
        dst = np.empty(max(ncol * k, 1), np.float64)
        self.L.check(self.lib.sdg_topk_block(self.h, D.ctypes.data, nrow, ncol, int(k),
                                             int(decreasing), sr.ctypes.data, idx.ctypes.data,
                                             dst.ctypes.data))
        return (idx[:ncol * k].reshape(k, ncol).T.copy(), dst[:ncol * k].reshape(k, ncol).T.copy())

    def topk_rows_accum(self, D, k, decreasing, best_idx, best_val, col_offset, self_col):
        D = np.asfortranarray(D, dtype=np.float64)
        nrow, ncol = D.shape
        bi = np.asfortranarray(best_idx, dtype=np.int32).copy(order="F")
        bv = np.asfortranarray(best_val, dtype=np.float64).copy(order="F")
        sc = np.ascontiguousarray(self_col, dtype=np.int32)
        self.L.check(self.lib.sdg_topk_rows_accum(self.h, D.ctypes.data, nrow, ncol, int(k),
                                                  int(decreasing), bi.ctypes.data, bv.ctypes.data,
                                                  int(col_offset), sc.ctypes.data))
        return bi, bv

    def snn_jaccard(self, idx, include_self=True):
        M = np.asfortranarray(idx, dtype=np.int32)
        n, k = M.shape
        w = np.empty(max(n * k, 1), np.float64)
        self.L.check(self.lib.sdg_snn_jaccard(self.h, M.ctypes.data, n, k, int(include_self),
                                              w.ctypes.data))
        return w[:n * k].reshape(k, n).T.copy()

    def snn_graph(self, idx, include_self=True, prune=0.0, symmetrise=True):
        M = np.asfortranarray(idx, dtype=np.int32)
        n, k = M.shape
        nnz = np.zeros(1, np.int64)
        self.L.check(self.lib.sdg_snn_graph(self.h, M.ctypes.data, n, k, int(include_self),
                                            float(prune), int(symmetrise), nnz.ctypes.data, None,
                                            None, None))
        m = int(nnz[0])
        p = np.empty(n + 1, np.int32)
        i = np.empty(max(m, 1), np.int32)
        x = np.empty(max(m, 1), np.float64)
        self.L.check(self.lib.sdg_snn_graph(self.h, M.ctypes.data, n, k, int(include_self),
                                            float(prune), int(symmetrise), nnz.ctypes.data,
                                            p.ctypes.data, i.ctypes.data, x.ctypes.data))
        return p, i[:m], x[:m]
