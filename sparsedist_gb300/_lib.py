"""ctypes binding of libsdgpu.so (the C ABI declared in include/sdgpu.h).

The library is the only compute path: if it is missing, or no CUDA device is
present, every call raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsdgpu.so")

SDG_OK = 0
STATUS_NAMES = {-1: "SDG_E_ARG", -2: "SDG_E_NONFINITE", -3: "SDG_E_ROWS", -4: "SDG_E_NOCAND",
                -5: "SDG_E_NOMEM", -6: "SDG_E_INDEX", -7: "SDG_E_CUDA", -8: "SDG_E_UNSUPPORTED",
                -9: "SDG_E_CANCELLED"}
WARN_CLAMP_FWD = 1
WARN_CLAMP_REV = 2

NA_INTEGER = np.int32(-(2 ** 31))
NA_REAL_BITS = np.uint64(0x7FF00000000007A2)

EXPORTED = ["sdg_version", "sdg_last_error", "sdg_ctx_create", "sdg_ctx_destroy", "sdg_ctx_cancel",
            "sdg_ctx_reset_cancel", "sdg_dist_cross", "sdg_dist", "sdg_topk_block", "sdg_topk_rows_accum",
            "sdg_snn_jaccard", "sdg_knn", "sdg_knn_cross", "sdg_snn_graph", "sdg_matrix_upload",
            "sdg_matrix_free", "sdg_knn_resident", "sdg_knn_resident_device", "sdg_ctx_set_stream",
            "sdg_last_stats", "sdg_ctx_set_engine", "sdg_debug_stall_tc", "sdg_kernel_time", "sdg_knn_block",
            "sdg_server_create", "sdg_server_submit", "sdg_server_wait", "sdg_server_result",
            "sdg_server_cancel", "sdg_server_stats", "sdg_server_destroy",
            "sdg_matrix_upload_device", "sdg_dense_upload", "sdg_dense_free", "sdg_dense_knn_block",
            "sdg_dense_knn_query", "sdg_server_create_dense", "sdg_server_submit_dense",
            "sdg_knn_cross_batch",
            "sdg_snn_graph_shared"]


class SdgError(RuntimeError):
    """A failure reported by libsdgpu.so; ``code`` is the sdg_status value."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code
        self.status = STATUS_NAMES.get(code, str(code))


class CSC(C.Structure):
    _fields_ = [("nrow", C.c_int32), ("ncol", C.c_int32),
                ("p", C.POINTER(C.c_int32)), ("i", C.POINTER(C.c_int32)),
                ("x", C.POINTER(C.c_double))]


_lib = None
_lib_lock = threading.Lock()


def load() -> C.CDLL:
    """Loads libsdgpu.so; raises if it has not been built."""
    global _lib
    with _lib_lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError("libsdgpu.so is not built (run `python -m sparsedist_gb300.build`); "
                                  "there is no CPU fallback")
            lib = C.CDLL(LIB_PATH)
            v = C.c_void_p
            lib.sdg_last_error.argtypes = [C.c_char_p, C.c_size_t]
            lib.sdg_ctx_create.argtypes = [C.c_int, C.POINTER(v)]
            lib.sdg_ctx_destroy.argtypes = [v]
            lib.sdg_ctx_cancel.argtypes = [v]
            lib.sdg_ctx_reset_cancel.argtypes = [v]
            lib.sdg_ctx_set_engine.argtypes = [v, C.c_int]
            lib.sdg_debug_stall_tc.argtypes = [C.c_int]
            lib.sdg_last_stats.argtypes = [v, v, C.c_int]
            lib.sdg_dist_cross.argtypes = [v, C.c_int, C.c_int, v, v, v]
            lib.sdg_dist.argtypes = [v, C.c_int, C.c_int, v, C.c_int, C.c_int, v]
            lib.sdg_topk_block.argtypes = [v, v, C.c_int64, C.c_int64, C.c_int, C.c_int, v, v, v]
            lib.sdg_topk_rows_accum.argtypes = [v, v, C.c_int64, C.c_int64, C.c_int, C.c_int, v, v,
                                                C.c_int32, v]
            lib.sdg_snn_jaccard.argtypes = [v, v, C.c_int32, C.c_int32, C.c_int, v]
            lib.sdg_snn_graph_shared.argtypes = [v, v, C.c_int32, C.c_int32, C.c_int, C.c_double,
                                                 v, v, v, v]
            lib.sdg_snn_graph.argtypes = [v, v, C.c_int32, C.c_int32, C.c_int, C.c_double, C.c_int,
                                          v, v, v, v]
            lib.sdg_knn.argtypes = [v, v, v, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, v, v, v, v]
            lib.sdg_knn_cross.argtypes = [v, v, v, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.c_int, v, v, v, v, v, v, v]
            lib.sdg_matrix_upload.argtypes = [v, v, C.POINTER(v)]
            lib.sdg_matrix_free.argtypes = [v]
            lib.sdg_knn_resident.argtypes = [v, v, v, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                             v, v, v, v]
            lib.sdg_knn_resident_device.argtypes = lib.sdg_knn_resident.argtypes
            lib.sdg_ctx_set_stream.argtypes = [v, v]
            lib.sdg_dense_upload.argtypes = [v, v, C.c_int32, C.c_int64, C.POINTER(v)]
            lib.sdg_dense_free.argtypes = [v]
            lib.sdg_dense_knn_block.argtypes = [v, v, C.c_int64, C.c_int64, C.c_int, C.c_int, C.c_int,
                                                v, v, C.c_int, v, v]
            lib.sdg_dense_knn_query.argtypes = [v, v, v, C.c_int32, C.c_int64, C.c_int, C.c_int, C.c_int,
                                                v, v, C.c_int, v, v]
            lib.sdg_matrix_upload_device.argtypes = [v, C.c_int32, C.c_int32, v, v, v, C.POINTER(v)]
            lib.sdg_server_create.argtypes = [v, v, C.c_int, C.c_int, C.c_int64, v, C.c_int,
                                              C.POINTER(v)]
            lib.sdg_server_submit.argtypes = [v, v, C.c_int, C.c_int, C.c_int, C.c_int, v]
            lib.sdg_knn_cross_batch.argtypes = [v, C.c_int, v, v, v, v, v, C.c_int, v, v, v, v, v, v, v, v, v, v]
            lib.sdg_server_create_dense.argtypes = [v, v, C.c_int, C.c_int, C.c_int64, C.POINTER(v)]
            lib.sdg_server_submit_dense.argtypes = [v, v, C.c_int32, C.c_int32, C.c_int, C.c_int, v]
            lib.sdg_server_wait.argtypes = [v, C.c_int64, C.c_int]
            lib.sdg_server_result.argtypes = [v, C.c_int64, v, v, v, v]
            lib.sdg_server_cancel.argtypes = [v, C.c_int64]
            lib.sdg_server_stats.argtypes = [v, v, C.c_int]
            lib.sdg_server_destroy.argtypes = [v]
            lib.sdg_knn_block.argtypes = [v, v, v, C.c_int64, C.c_int64, C.c_int, C.c_int, C.c_int,
                                          C.c_int, C.c_int, v, v, C.c_int, v, v]
            lib.sdg_kernel_time.argtypes = [v, v, v]
            _lib = lib
    return _lib


def last_error() -> str:
    lib = load()
    buf = C.create_string_buffer(4096)
    lib.sdg_last_error(buf, 4096)
    return buf.value.decode()


def check(status: int):
    if status != SDG_OK:
        raise SdgError(status, last_error())


class Context:
    """An sdg_ctx: one CUDA stream on one device."""

    def __init__(self, device: int = -1):
        lib = load()
        h = C.c_void_p()
        check(lib.sdg_ctx_create(int(device), C.byref(h)))
        self.handle = h
        self.lib = lib

    def close(self):
        if self.handle:
            self.lib.sdg_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_engine(self, engine: int):
        check(self.lib.sdg_ctx_set_engine(self.handle, int(engine)))

    def set_stream(self, stream_ptr):
        """Launch on the caller's CUDA stream (an integer cudaStream_t, e.g.
        torch.cuda.current_stream().cuda_stream); None restores the own stream."""
        check(self.lib.sdg_ctx_set_stream(self.handle, C.c_void_p(stream_ptr) if stream_ptr else None))

    def cancel(self):
        check(self.lib.sdg_ctx_cancel(self.handle))

    def reset_cancel(self):
        check(self.lib.sdg_ctx_reset_cancel(self.handle))

    def kernel_time(self):
        """(total ms, launches) of the bounding kernel since the last call."""
        ms = np.zeros(1, np.float64)
        n = np.zeros(1, np.int64)
        check(self.lib.sdg_kernel_time(self.handle, ms.ctypes.data, n.ctypes.data))
        return float(ms[0]), int(n[0])

    def stats(self):
        out = np.zeros(8, np.int64)
        check(self.lib.sdg_last_stats(self.handle, out.ctypes.data, 8))
        return {"pairs_screened": int(out[0]), "pairs_exact": int(out[1]),
                "overflow_queries": int(out[2]), "kernels": int(out[3]),
                "screen_us": int(out[4]), "device_us": int(out[5]), "tensor_flops": int(out[6])}


_tls = threading.local()


def default_context() -> Context:
    ctx = getattr(_tls, "ctx", None)
    if ctx is None:
        ctx = Context()
        _tls.ctx = ctx
    return ctx


class HeldCSC:
    """Keeps contiguous int32/float64 CSC arrays alive behind a CSC struct."""

    def __init__(self, nrow, ncol, p, i, x):
        self.p = np.ascontiguousarray(p, dtype=np.int32)
        self.i = np.ascontiguousarray(i, dtype=np.int32)
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.nrow, self.ncol = int(nrow), int(ncol)
        self.s = CSC(self.nrow, self.ncol, self.p.ctypes.data_as(C.POINTER(C.c_int32)),
                     self.i.ctypes.data_as(C.POINTER(C.c_int32)),
                     self.x.ctypes.data_as(C.POINTER(C.c_double)))

    @property
    def ref(self):
        return C.byref(self.s)


class Resident:
    """An sdg_matrix: a CSC matrix kept in device memory (sdg_matrix_upload)."""

    def __init__(self, ctx: Context, nrow, ncol, p, i, x):
        self.ctx = ctx
        held = HeldCSC(nrow, ncol, p, i, x)
        h = C.c_void_p()
        check(ctx.lib.sdg_matrix_upload(ctx.handle, held.ref, C.byref(h)))
        self.handle = h
        self.nrow, self.ncol = int(nrow), int(ncol)

    @classmethod
    def from_device(cls, ctx: Context, nrow, ncol, d_p, d_i, d_x):
        """From dgCMatrix slots in device memory (torch tensors: int32 p / i,
        float64 x); copied device to device."""
        self = cls.__new__(cls)
        self.ctx = ctx
        h = C.c_void_p()
        check(ctx.lib.sdg_matrix_upload_device(ctx.handle, int(nrow), int(ncol), d_p.data_ptr(),
                                               d_i.data_ptr(), d_x.data_ptr(), C.byref(h)))
        self.handle = h
        self.nrow, self.ncol = int(nrow), int(ncol)
        return self

    def free(self):
        if self.handle:
            self.ctx.lib.sdg_matrix_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Server:
    """sdg_server: continuous-batching kNN service against a resident reference."""

    def __init__(self, ctx: Context, ref, workers=2, max_slots=64,
                 mem_budget=120 << 30, methods=(1,), dense=False):
        """ref: a Resident (sparse reference) or, with dense=True, the handle
        of an sdg_dense (sdg_dense_upload)."""
        self.ctx, self.ref = ctx, ref
        h = C.c_void_p()
        if dense:
            check(ctx.lib.sdg_server_create_dense(ctx.handle, ref, int(workers), int(max_slots),
                                                  int(mem_budget), C.byref(h)))
        else:
            m = np.ascontiguousarray(methods, dtype=np.int32)
            check(ctx.lib.sdg_server_create(ctx.handle, ref.handle, int(workers), int(max_slots),
                                            int(mem_budget), m.ctypes.data, len(m), C.byref(h)))
        self.handle = h
        self.lib = ctx.lib
        self._held = {}

    def submit_dense(self, Q, method=1, k=10):
        """Q: d x nq FP32 query columns (host memory, column-major: a
        C-contiguous (nq, d) array is read as its transpose)."""
        Q = np.asarray(Q)
        if Q.dtype != np.float32 or not Q.flags.c_contiguous:
            raise ValueError("Q must be a C-contiguous float32 (nq, d) array")
        nq, d = Q.shape
        rid = C.c_int64()
        check(self.lib.sdg_server_submit_dense(self.handle, Q.ctypes.data, int(d), int(nq), int(method),
                                               int(k), C.byref(rid)))
        self._held[rid.value] = (nq, k)
        return rid.value

    def submit(self, nrow, ncol, p, i, x, method=1, dist=True, k=10, drop_degenerate=True):
        held = HeldCSC(nrow, ncol, p, i, x)
        rid = C.c_int64()
        check(self.lib.sdg_server_submit(self.handle, held.ref, int(method), int(bool(dist)), int(k),
                                         int(bool(drop_degenerate)), C.byref(rid)))
        self._held[rid.value] = (ncol, k)
        return rid.value

    def wait(self, rid, timeout_ms=-1):
        st = self.lib.sdg_server_wait(self.handle, C.c_int64(rid), int(timeout_ms))
        if st < 0:
            check(st)
        return st == 0

    def result(self, rid):
        ncol, k = self._held.pop(rid)
        idx = np.empty(ncol * k, np.int32)
        dst = np.empty(ncol * k, np.float64)
        ke, fl = C.c_int(), C.c_int()
        check(self.lib.sdg_server_result(self.handle, C.c_int64(rid), idx.ctypes.data,
                                         dst.ctypes.data, C.byref(ke), C.byref(fl)))
        e = ke.value
        return idx[:ncol * e].reshape(e, ncol).T.copy(), dst[:ncol * e].reshape(e, ncol).T.copy(), fl.value

    def cancel(self, rid):
        """True when the request was cancelled before it started (its result
        then raises SDG_E_CANCELLED); False when it is already running."""
        st = self.lib.sdg_server_cancel(self.handle, C.c_int64(rid))
        if st < 0:
            check(st)
        return st == 0

    def stats(self):
        out = np.zeros(9, np.float64)
        check(self.lib.sdg_server_stats(self.handle, out.ctypes.data, 9))
        keys = ["completed", "columns", "p50_s", "p99_s", "mean_s", "columns_per_s", "batches",
                "bytes_admitted", "waiting"]
        return dict(zip(keys, out.tolist()))

    def close(self):
        if self.handle:
            self.lib.sdg_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def knn_cross_batch(ctx, problems, drop_degenerate=True):
    """sdg_knn_cross_batch over a list of (X, Y, method_code, dist, k) with X, Y
    scipy CSC matrices.  Returns one dict per problem: forward / reverse
    (idx, dist) as (n, k_eff) arrays, flags, status (0 or the sdg_status) and
    the engines chosen for the two directions."""
    n = len(problems)
    held = [(HeldCSC(X.shape[0], X.shape[1], X.indptr, X.indices, X.data),
             HeldCSC(Y.shape[0], Y.shape[1], Y.indptr, Y.indices, Y.data)) for X, Y, _, _, _ in problems]
    Xs = (CSC * max(n, 1))(*[h[0].s for h in held])
    Ys = (CSC * max(n, 1))(*[h[1].s for h in held])
    meth = np.array([p[2] for p in problems] or [0], np.int32)
    dist = np.array([int(bool(p[3])) for p in problems] or [0], np.int32)
    ks = np.array([p[4] for p in problems] or [1], np.int32)
    outs = []
    for (X, Y, _, _, k) in problems:
        outs.append((np.empty(max(X.shape[1] * k, 1), np.int32), np.empty(max(X.shape[1] * k, 1), np.float64),
                     np.empty(max(Y.shape[1] * k, 1), np.int32), np.empty(max(Y.shape[1] * k, 1), np.float64)))
    ptrs = [(C.c_void_p * max(n, 1))(*[o[j].ctypes.data for o in outs]) for j in range(4)]
    kf, kr, fl, st = (np.zeros(max(n, 1), np.int32) for _ in range(4))
    eng = np.zeros(2 * max(n, 1), np.int32)
    secs = np.zeros(3, np.float64)
    rc = ctx.lib.sdg_knn_cross_batch(ctx.handle, n, C.cast(Xs, C.c_void_p), C.cast(Ys, C.c_void_p),
                                     meth.ctypes.data, dist.ctypes.data, ks.ctypes.data, int(bool(drop_degenerate)),
                                     C.cast(ptrs[0], C.c_void_p), C.cast(ptrs[1], C.c_void_p),
                                     C.cast(ptrs[2], C.c_void_p), C.cast(ptrs[3], C.c_void_p), kf.ctypes.data,
                                     kr.ctypes.data, fl.ctypes.data, st.ctypes.data, eng.ctypes.data,
                                     secs.ctypes.data)
    res = []
    for p, (X, Y, _, _, k) in enumerate(problems):
        nx, ny, a, b = X.shape[1], Y.shape[1], int(kf[p]), int(kr[p])
        fi, fd, ri, rd = outs[p]
        # (n, k) views of the column-major results (the R layout), no copies
        res.append({"forward": (fi[:nx * a].reshape(a, nx).T, fd[:nx * a].reshape(a, nx).T),
                    "reverse": (ri[:ny * b].reshape(b, ny).T, rd[:ny * b].reshape(b, ny).T),
                    "flags": int(fl[p]), "status": int(st[p]), "engines": (int(eng[2 * p]), int(eng[2 * p + 1]))})
    knn_cross_batch.engine_seconds = secs.tolist()
    return rc, res


def na_real(shape) -> np.ndarray:
    return np.full(shape, NA_REAL_BITS, dtype=np.uint64).view(np.float64)
