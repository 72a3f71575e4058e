"""mf_columns_sum_noalloc: column sums for callers that cannot allocate.

The entry point serves code that must not allocate device memory where it
needs the sums: code whose device memory all comes from its own arena or
another framework's allocator, a process whose allocation budget is spent,
or a latency-critical loop where cudaMalloc/cudaFree would stall the device.
Its scratch is a fixed array inside the library, so it takes plain device
pointers and a stream, and no context.

These tests call it through the C ABI and check it against mf_columns_sum
(which takes its scratch from a context): the same kernel, grid and combine
order, so the sums must be equal bit for bit. They also check both against
the exactly rounded column sums of the host data (math.fsum), within the bar
the other column-sum tests use (1e-13 of the sum of absolute values), and
that a call allocates nothing (the context's allocation count and the
device's free memory are unchanged across it). Two calls in a row with
different shapes and element types check that the shared scratch carries
nothing over from one call to the next. The file runs last (its name sorts
last) and sets up its own context, so it passes alone in a fresh process and
after the other tests alike.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_COLS = 64  # the entry point's documented column limit


@pytest.fixture(scope="module")
def backend():
    from morefit_gb300.backend import CUDABackend
    b = CUDABackend(0)
    yield b
    b.close()


def _stream(backend):
    from morefit_gb300 import _lib as L
    s = C.c_void_p()
    L.check(L.lib.mf_context_stream(backend.handle, C.byref(s)))
    return s


def _device_sums(backend, ncols):
    from morefit_gb300 import _lib as L
    b = L.c_buf()
    L.check(L.lib.mf_buffer_alloc(backend.handle, ncols * 8, C.byref(b)))
    return b


def _noalloc(backend, cols, sums_buf, ncols):
    """One call of the entry point on the context's stream; returns the sums."""
    from morefit_gb300 import _lib as L
    L.check(L.lib.mf_columns_sum_noalloc(L.lib.mf_buffer_device_ptr(cols.buf), cols.elem, ncols, cols.n,
                                         cols.stride, L.lib.mf_buffer_device_ptr(sums_buf), _stream(backend)))
    out = np.zeros(ncols)
    # mf_buffer_d2h copies on the same stream, after the sums are written.
    L.check(L.lib.mf_buffer_d2h(sums_buf, 0, out.ctypes.data, ncols * 8))
    return out


def _with_scratch(cols, ncols):
    from morefit_gb300 import _lib as L
    out = np.zeros(ncols)
    L.check(L.lib.mf_columns_sum(cols.buf, cols.elem, ncols, cols.n, cols.stride, L.dptr(out)))
    return out


def _upload(backend, elem, ncols, n, seed):
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import DeviceColumns
    host = np.random.default_rng(seed).normal(0.3, 2.0, size=(ncols, n))
    if elem == L.MF_F32:
        host = host.astype(np.float32)
    cols = DeviceColumns(backend, elem)
    cols.upload(host)
    h64 = host.astype(np.float64)
    return cols, np.abs(h64).sum(axis=1), np.array([math.fsum(r) for r in h64])


def _allocated(backend):
    from morefit_gb300 import _lib as L
    v = C.c_uint64()
    L.check(L.lib.mf_context_allocated(backend.handle, C.byref(v)))
    return v.value


def _device_free():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


def test_noalloc_matches_columns_sum_twice_in_a_row(backend):
    from morefit_gb300 import _lib as L
    # First call: FP64, 14 columns (the P-wave block width), a full grid.
    a, scale_a, exact_a = _upload(backend, L.MF_F64, 14, 1_000_003, seed=11)
    # Second call: FP32, the full 64 columns, a ragged n that gives a smaller grid.
    b, scale_b, exact_b = _upload(backend, L.MF_F32, MAX_COLS, 77_777, seed=12)
    sums_a, sums_b = _device_sums(backend, 14), _device_sums(backend, MAX_COLS)
    try:
        got_a = _noalloc(backend, a, sums_a, 14)
        got_b = _noalloc(backend, b, sums_b, MAX_COLS)
        ref_a, ref_b = _with_scratch(a, 14), _with_scratch(b, MAX_COLS)
        assert np.array_equal(got_a, ref_a), (got_a, ref_a, np.abs(got_a - ref_a) / scale_a)
        assert np.array_equal(got_b, ref_b), (got_b, ref_b, np.abs(got_b - ref_b) / scale_b)
        assert np.all(np.abs(got_a - exact_a) <= 1e-13 * scale_a), (got_a, exact_a)
        assert np.all(np.abs(got_b - exact_b) <= 1e-13 * scale_b), (got_b, exact_b)
        # Same data again after the other call: the same sums, and no allocation.
        before = (_allocated(backend), _device_free())
        again = _noalloc(backend, a, sums_a, 14)
        assert (_allocated(backend), _device_free()) == before
        assert np.array_equal(again, got_a)
    finally:
        for buf in (sums_a, sums_b):
            L.check(L.lib.mf_buffer_free(buf))
        a.free()
        b.free()


def test_noalloc_rejects_too_many_columns(backend):
    from morefit_gb300 import _lib as L
    a, _, _ = _upload(backend, L.MF_F64, 1, 1000, seed=13)
    sums = _device_sums(backend, 1)
    try:
        rc = L.lib.mf_columns_sum_noalloc(L.lib.mf_buffer_device_ptr(a.buf), L.MF_F64, MAX_COLS + 1, 1000,
                                          a.stride, L.lib.mf_buffer_device_ptr(sums), _stream(backend))
        assert rc == L.MF_ERR_INVALID
        assert b"ncols must be 1..64" in L.lib.mf_last_error()
    finally:
        L.check(L.lib.mf_buffer_free(sums))
        a.free()
