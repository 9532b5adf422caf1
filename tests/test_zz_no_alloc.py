"""xtt_dot_noalloc: the TT dot product for callers that cannot allocate device
memory (their device memory is owned by another allocator, or cudaMalloc /
cudaFree are not acceptable on their path). The caller owns every buffer; the
entry point keeps its intermediates in a fixed array inside the library.

Checked through the C ABI against xtt_dot (which allocates scratch through its
context), on two calls in a row and on a second pair of tensors, and the
capacity limit is rejected before any launch; after a warm-up call, further calls
leave the device's free memory unchanged (they allocate nothing). This file is
collected last so a failure here cannot hide failures elsewhere.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def ctx():
    from xerus_gb300 import build
    build.build()
    import xerus_gb300 as xg
    return xg.Context(0)


def _device_copy(t):
    flat = torch.from_numpy(t.get_flat()).cuda()
    return flat, np.array(t.all_ranks(), dtype=np.int64)


def _noalloc_dot(lib, dims, x, y, stream):
    xd, xr = _device_copy(x)
    yd, yr = _device_copy(y)
    out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    d = np.array(dims, dtype=np.int64)
    p = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    rc = lib.xtt_dot_noalloc(len(dims), p(d), p(xr), ctypes.c_void_p(xd.data_ptr()), p(yr),
                             ctypes.c_void_p(yd.data_ptr()), ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))
    assert rc == 0, lib.xtt_last_error()
    torch.cuda.synchronize()
    return float(out.item())


def test_noalloc_dot_matches_dot_twice(ctx):
    import xerus_gb300 as xg
    lib = xg._lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    xg.seed(11)
    dims = [4, 3, 4, 2, 4, 3, 4, 2]
    x = xg.TTTensor.random(dims, [4, 12, 16, 8, 16, 12, 4], ctx=ctx)
    y = xg.TTTensor.random(dims, [3, 9, 20, 8, 20, 9, 3], ctx=ctx)
    want = xg.dot(x, y)
    for _ in range(2):
        got = _noalloc_dot(lib, dims, x, y, stream)
        assert abs(got - want) <= 1e-12 * abs(want)
    # a different shape afterwards: nothing of the previous calls may leak in
    dims2 = [16, 2, 5]
    u = xg.TTTensor.random(dims2, [16, 10], ctx=ctx)
    v = xg.TTTensor.random(dims2, [7, 5], ctx=ctx)
    want2 = xg.dot(u, v)
    for _ in range(2):
        got2 = _noalloc_dot(lib, dims2, u, v, stream)
        assert abs(got2 - want2) <= 1e-12 * abs(want2)


def test_noalloc_dot_rejects_sizes_beyond_the_limit(ctx):
    import xerus_gb300 as xg
    lib = xg._lib.load()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    ptr = ctypes.c_void_p(buf.data_ptr())
    p = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    dims = np.array([17, 2], dtype=np.int64)
    ranks = np.array([1, 1, 1], dtype=np.int64)
    assert lib.xtt_dot_noalloc(2, p(dims), p(ranks), ptr, p(ranks), ptr, ptr, None) == 6  # XTT_ERR_CAPACITY
    assert b"limit" in lib.xtt_last_error()
    dims = np.array([2, 2], dtype=np.int64)
    big = np.array([1, 129, 1], dtype=np.int64)
    assert lib.xtt_dot_noalloc(2, p(dims), p(big), ptr, p(ranks), ptr, ptr, None) == 6
    host = np.zeros(8)
    hptr = ctypes.c_void_p(host.ctypes.data)
    assert lib.xtt_dot_noalloc(2, p(dims), p(ranks), hptr, p(ranks), ptr, ptr, None) == 1  # host memory refused


def test_noalloc_dot_allocates_nothing(ctx):
    """After a warm-up call (which looks up the array's address and loads the kernels),
    repeated calls leave the device's free memory exactly unchanged."""
    import xerus_gb300 as xg
    lib = xg._lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    xg.seed(13)
    dims = [4, 4, 4, 4, 4, 4]
    x = xg.TTTensor.random(dims, [4, 16, 32, 16, 4], ctx=ctx)
    y = xg.TTTensor.random(dims, [4, 8, 24, 8, 4], ctx=ctx)
    want = xg.dot(x, y)
    xd, xr = _device_copy(x)
    yd, yr = _device_copy(y)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    d = np.array(dims, dtype=np.int64)
    p = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
    args = (len(dims), p(d), p(xr), ctypes.c_void_p(xd.data_ptr()), p(yr), ctypes.c_void_p(yd.data_ptr()),
            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))
    assert lib.xtt_dot_noalloc(*args) == 0, lib.xtt_last_error()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        assert lib.xtt_dot_noalloc(*args) == 0, lib.xtt_last_error()
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    assert abs(float(out.item()) - want) <= 1e-12 * abs(want)
