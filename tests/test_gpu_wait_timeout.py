"""The fused tensor-core screens' bounded waits, made to run out on purpose.

sdg_debug_stall_tc(1) makes the next launch's MMA issuer wait on a pipeline
phase that nothing completes (a flag nothing sets).  The wait gives up after
its 1 s limit, the CTA's other roles leave their loops, every issued TMA copy
and MMA is drained and TMEM is freed before the kernel returns; the call must
fail with SDG_E_CUDA and a "timed out" message, and the next call on the same
context must succeed with the oracle's result.  No fault, trap or unbounded
wait is involved: the kernel returns by itself."""
import ctypes as C

import pytest
import scipy.sparse as sp

from backends import OracleBackend, make_x, same_bits

pytestmark = pytest.mark.gpu

SDG_E_CUDA = -7                 # include/sdgpu.h


def test_dense_screen_wait_runs_out_and_context_recovers():
    import torch
    from sparsedist_gb300 import _lib, synth
    from test_gpu_dense import dense_knn
    X = synth.dense_embeddings(d=64, n=3000, centres=20, seed=5)
    ctx = _lib.Context()
    h = C.c_void_p()
    _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), 64, 3000, C.byref(h)))
    try:
        _lib.check(ctx.lib.sdg_debug_stall_tc(1))
        with pytest.raises(_lib.SdgError) as ei:
            dense_knn(ctx, h, 0, 3000, 1, 15, 0)
        assert ei.value.code == SDG_E_CUDA and "timed out" in str(ei.value)
        got = dense_knn(ctx, h, 0, 3000, 1, 15, 0)
    finally:
        ctx.lib.sdg_debug_stall_tc(0)
        ctx.lib.sdg_dense_free(h)
    want = OracleBackend().knn(sp.csc_matrix(X.double().cpu().numpy().T), k=15, method="cosine")
    assert same_bits(got[0], want[0]) and same_bits(got[1], want[1])
    torch.cuda.synchronize()


def test_sparse_screen_wait_runs_out_and_context_recovers(gpu):
    from sparsedist_gb300 import _lib
    X = make_x(600, 900, 0.05, 31)
    gpu.set_engine(3)
    try:
        _lib.check(gpu.lib.sdg_debug_stall_tc(1))
        with pytest.raises(_lib.SdgError) as ei:
            gpu.knn(X, k=12, method="cosine")
        assert ei.value.code == SDG_E_CUDA and "timed out" in str(ei.value)
        got = gpu.knn(X, k=12, method="cosine")
    finally:
        gpu.lib.sdg_debug_stall_tc(0)
        gpu.set_engine(0)
    want = OracleBackend().knn(X, k=12, method="cosine")
    assert same_bits(got[0], want[0]) and same_bits(got[1], want[1])


def test_stall_hook_rejects_negative_counts():
    from sparsedist_gb300 import _lib
    lib = _lib.load()
    assert lib.sdg_debug_stall_tc(-1) != 0
    assert lib.sdg_debug_stall_tc(0) == 0


def test_dense_screen_pair_wait_runs_out():
    # the CTA-pair form of the dense kernel (mode 3) the same way
    import torch
    from sparsedist_gb300 import _lib, synth
    from test_gpu_dense import dense_knn
    X = synth.dense_embeddings(d=64, n=3000, centres=20, seed=6)
    ctx = _lib.Context()
    h = C.c_void_p()
    _lib.check(ctx.lib.sdg_dense_upload(ctx.handle, X.data_ptr(), 64, 3000, C.byref(h)))
    try:
        _lib.check(ctx.lib.sdg_debug_stall_tc(1))
        with pytest.raises(_lib.SdgError) as ei:
            dense_knn(ctx, h, 0, 3000, 1, 15, 3)
        assert ei.value.code == SDG_E_CUDA and "timed out" in str(ei.value)
        got = dense_knn(ctx, h, 0, 3000, 1, 15, 3)
    finally:
        ctx.lib.sdg_debug_stall_tc(0)
        ctx.lib.sdg_dense_free(h)
    want = OracleBackend().knn(sp.csc_matrix(X.double().cpu().numpy().T), k=15, method="cosine")
    assert same_bits(got[0], want[0]) and same_bits(got[1], want[1])
    torch.cuda.synchronize()
