"""sdg_snn_jaccard_noalloc: the SNN weights for callers that cannot allocate
device memory on their call path (a host framework that owns the GPU's memory
through its own allocator, or a thread that must not call cudaMalloc /
cudaFree because they synchronise the device).  The entry point takes device
pointers and keeps its scratch in a fixed array inside the library.

Checked through the C ABI against the allocating entry point
(sdg_snn_jaccard): bit for bit, the tolerance every SNN test here uses, on two
calls in a row with different inputs (the shared scratch keeps the previous
call's contents).  This file is collected last so that a run stopping at the
first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NA = np.int32(-(2 ** 31))


def knn_like(n, k, seed):
    rng = np.random.default_rng(seed)
    idx = rng.integers(1, n + 1, size=(n, k)).astype(np.int32)
    idx[rng.random((n, k)) < 0.05] = NA            # padding
    idx[:, 0] = np.where(rng.random(n) < 0.1, np.arange(1, n + 1), idx[:, 0])  # explicit self
    idx[:, 1] = np.where(rng.random(n) < 0.1, idx[:, 2], idx[:, 1])            # duplicates
    return np.asfortranarray(idx)


def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    from sparsedist_gb300 import _lib
    lib = _lib.load()
    fn = lib.sdg_snn_jaccard_noalloc
    fn.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int, C.c_void_p, C.c_void_p]
    ctx = _lib.Context()
    stream = torch.cuda.current_stream().cuda_stream
    for call, (n, k, inc, seed) in enumerate([(3000, 15, 1, 1), (1700, 9, 0, 2)]):
        idx = knn_like(n, k, seed)
        want = np.empty(n * k, np.float64)
        _lib.check(ctx.lib.sdg_snn_jaccard(ctx.handle, idx.ctypes.data, n, k, inc,
                                           want.ctypes.data))
        d_idx = torch.from_numpy(idx.reshape(-1, order="F").copy()).cuda()
        d_w = torch.full((n * k,), -1.0, dtype=torch.float64, device="cuda")
        _lib.check(fn(d_idx.data_ptr(), n, k, inc, d_w.data_ptr(), stream))
        torch.cuda.synchronize()
        got = d_w.cpu().numpy()
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), "call %d" % call


def test_noalloc_rejects_bad_input_then_recovers():
    torch = pytest.importorskip("torch")
    from sparsedist_gb300 import _lib
    lib = _lib.load()
    fn = lib.sdg_snn_jaccard_noalloc
    fn.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int, C.c_void_p, C.c_void_p]
    stream = torch.cuda.current_stream().cuda_stream
    d_w = torch.empty(16, dtype=torch.float64, device="cuda")
    bad = torch.tensor([1, 99, 2, 3], dtype=torch.int32, device="cuda")   # 4 x 1, 99 > n
    st = fn(bad.data_ptr(), 4, 1, 1, d_w.data_ptr(), stream)
    assert st == -6 and "1-based row indices" in _lib.last_error()
    # beyond the fixed scratch: rejected before any device work
    st = fn(bad.data_ptr(), 4_000_000, 1, 1, d_w.data_ptr(), stream)
    assert st == -8 and "scratch" in _lib.last_error()
    # the flag is cleared by the next call: S = {0,1}, {0,1}, {0,2}, {1,3}
    good = torch.tensor([2, 1, 1, 2], dtype=torch.int32, device="cuda")
    _lib.check(fn(good.data_ptr(), 4, 1, 1, d_w.data_ptr(), stream))
    torch.cuda.synchronize()
    assert d_w[:4].cpu().numpy().tolist() == [1.0, 1.0, 1 / 3, 1 / 3]
