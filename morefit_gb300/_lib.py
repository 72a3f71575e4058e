"""ctypes binding of the C ABI in include/morefit_cuda.h.

The native library is required: importing this module without a built
``libmorefit_cuda.so`` raises ImportError (run ``__graft_entry__.build()`` or
``python -m morefit_gb300.build``). There is no CPU fallback on the product
path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "_build" / "libmorefit_cuda.so"

MF_OK = 0
MF_ERR_INVALID = 1
MF_ERR_CUDA = 2
MF_ERR_NVRTC = 3
MF_ERR_PARSE = 4
MF_ERR_BUDGET = 5
MF_ERR_NO_DEVICE = 6
MF_ERR_UNSUPPORTED = 7
MF_ERR_TIMEOUT = 8
MF_ERR_NOT_READY = 9

MF_F64 = 0
MF_F32 = 1
MF_KERNEL_REDUCE = 0
MF_KERNEL_STORE = 1
MF_KERNEL_GENERATE = 2
MF_COLUMN_ALIGN = 64

_NAMES = {1: "INVALID", 2: "CUDA", 3: "NVRTC", 4: "PARSE", 5: "BUDGET", 6: "NO_DEVICE", 7: "UNSUPPORTED",
          8: "TIMEOUT", 9: "NOT_READY"}


class MFError(RuntimeError):
    """A C ABI call returned an MF_ERR_* status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"MF_ERR_{_NAMES.get(code, code)}: {message}")
        self.code = code


if not _LIB_PATH.exists():
    raise ImportError(f"native library {_LIB_PATH} is not built; run __graft_entry__.build()")

lib = C.CDLL(str(_LIB_PATH))

c_ctx = C.c_void_p
c_buf = C.c_void_p
c_ker = C.c_void_p
c_coal = C.c_void_p
c_char_pp = C.POINTER(C.c_char_p)
c_dbl_p = C.POINTER(C.c_double)


class KernelDesc(C.Structure):
    _fields_ = [
        ("name", C.c_char_p),
        ("kind", C.c_int),
        ("elem_type", C.c_int),
        ("n_inputs", C.c_uint32),
        ("input_names", c_char_pp),
        ("n_params", C.c_uint32),
        ("param_names", c_char_pp),
        ("n_outputs", C.c_uint32),
        ("exprs", c_char_pp),
        ("n_gen_dims", C.c_uint32),
        ("gen_dim_names", c_char_pp),
        ("gen_lo", c_dbl_p),
        ("gen_hi", c_dbl_p),
        ("maxprob", C.c_double),
        ("flags", C.c_uint32),
        ("vec", C.c_uint32),
        ("block", C.c_uint32),
        ("stages", C.c_uint32),
        ("param_defs", c_char_pp),
    ]


MF_FLAG_NATIVE_F64 = 1
MF_FLAG_F32_ARITH = 2
MF_FLAG_BULK_PIPELINE = 4


def _proto(name, restype, *args):
    f = getattr(lib, name)
    f.restype = restype
    f.argtypes = list(args)
    return f


_proto("mf_last_error", C.c_char_p)
_proto("mf_version", C.c_char_p)
_proto("mf_device_count", C.c_int, C.POINTER(C.c_int))
_proto("mf_context_set_resident", C.c_int, c_ctx, C.c_uint32)
_proto("mf_context_resident_stats", C.c_int, c_ctx, C.POINTER(C.c_int), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
       C.POINTER(C.c_int))
_proto("mf_compile_check_resident", C.c_int, C.c_void_p, C.c_uint32, C.POINTER(C.c_int), C.POINTER(C.c_int),
       C.c_char_p, C.c_size_t)
_proto("mf_device_properties", C.c_int, C.c_int, C.c_char_p, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int),
       C.POINTER(C.c_int))
_proto("mf_context_create", C.c_int, C.c_int, C.c_uint64, C.POINTER(c_ctx))
_proto("mf_context_destroy", C.c_int, c_ctx)
_proto("mf_context_allocated", C.c_int, c_ctx, C.POINTER(C.c_uint64))
_proto("mf_context_synchronize", C.c_int, c_ctx)
_proto("mf_buffer_alloc", C.c_int, c_ctx, C.c_uint64, C.POINTER(c_buf))
_proto("mf_buffer_free", C.c_int, c_buf)
_proto("mf_buffer_size", C.c_uint64, c_buf)
_proto("mf_buffer_device_ptr", C.c_void_p, c_buf)
_proto("mf_buffer_h2d", C.c_int, c_buf, C.c_uint64, C.c_void_p, C.c_uint64)
_proto("mf_buffer_d2h", C.c_int, c_buf, C.c_uint64, C.c_void_p, C.c_uint64)
_proto("mf_buffer_memset", C.c_int, c_buf, C.c_int)
_proto("mf_column_stride", C.c_uint64, C.c_uint64)
_proto("mf_events_upload", C.c_int, c_buf, C.c_int, C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint64)
_proto("mf_events_download", C.c_int, c_buf, C.c_int, C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint64)
_proto("mf_events_upload_f64_as", C.c_int, c_buf, C.c_int, c_dbl_p, C.c_uint32, C.c_uint64, C.c_uint64,
       C.c_uint64)
_proto("mf_kernel_build", C.c_int, c_ctx, C.POINTER(KernelDesc), C.POINTER(c_ker))
_proto("mf_kernel_free", C.c_int, c_ker)
_proto("mf_kernel_source", C.c_int, c_ker, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t))
_proto("mf_kernel_info", C.c_int, c_ker, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
       C.POINTER(C.c_int))
_proto("mf_kernel_reduce", C.c_int, c_ker, c_buf, C.c_uint64, C.c_uint64, c_dbl_p, C.c_uint32, c_dbl_p)
_proto("mf_kernel_reduce_async", C.c_int, c_ker, c_buf, C.c_uint64, C.c_uint64, c_dbl_p, C.c_uint32, c_buf,
       C.c_uint64)
_proto("mf_kernel_reduce_many", C.c_int, c_ker, C.c_uint32, C.POINTER(c_buf), C.POINTER(C.c_uint64),
       C.POINTER(C.c_uint64), c_dbl_p, C.c_uint32, c_buf)
_proto("mf_columns_sum", C.c_int, c_buf, C.c_int, C.c_uint32, C.c_uint64, C.c_uint64, c_dbl_p)
_proto("mf_columns_sum_noalloc", C.c_int, C.c_void_p, C.c_int, C.c_uint32, C.c_uint64, C.c_uint64, C.c_void_p,
       C.c_void_p)
_proto("mf_context_stream", C.c_int, c_ctx, C.POINTER(C.c_void_p))
_proto("mf_buffer_mark_modified", C.c_int, c_buf)
_proto("mf_expr_set_create", C.c_int, C.c_uint32, c_char_pp, C.c_uint32, c_char_pp, C.POINTER(C.c_void_p))
_proto("mf_expr_set_eval", C.c_int, C.c_void_p, C.c_uint32, c_dbl_p, c_dbl_p)
_proto("mf_expr_set_free", C.c_int, C.c_void_p)
_proto("mf_kernel_generate_segments", C.c_int, c_ker, C.POINTER(C.c_uint32), C.c_uint32, C.c_uint32, C.c_uint32,
       C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), c_dbl_p, C.c_uint32, c_dbl_p, c_buf, C.c_uint64, C.c_uint64)
_proto("mf_eval_expressions_batch", C.c_int, C.c_uint32, c_char_pp, C.c_uint32, c_dbl_p, C.c_uint32, c_char_pp,
       c_dbl_p)
_proto("mf_events_upload_async", C.c_int, c_buf, C.c_int, C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint64)
_proto("mf_buffer_d2h_async", C.c_int, c_buf, C.c_uint64, C.c_void_p, C.c_uint64)
_proto("mf_kernel_store_async", C.c_int, c_ker, c_buf, C.c_uint64, C.c_uint64, c_dbl_p, C.c_uint32, c_buf, C.c_uint64)
_proto("mf_kernel_read_layout", C.c_int, c_ker, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32))
_proto("mf_kernel_reduce_segments", C.c_int, c_ker, c_buf, C.c_uint64, C.c_uint32, C.POINTER(C.c_uint64),
       C.POINTER(C.c_uint32), c_dbl_p, C.c_uint32, c_dbl_p)
_proto("mf_kernel_reduce_segments_chunked", C.c_int, c_ker, c_buf, C.c_uint64, C.c_uint32, C.POINTER(C.c_uint64),
       C.POINTER(C.c_uint32), c_dbl_p, C.c_uint32, C.c_uint32, c_dbl_p)
_proto("mf_kernel_fallback_count", C.c_int, c_ker, C.POINTER(C.c_uint64))
_proto("mf_buffer_wrap_host", C.c_int, c_ctx, C.c_void_p, C.c_uint64, C.POINTER(c_buf))
_proto("mf_events_load_file", C.c_int, c_buf, C.c_int, C.c_uint64, C.c_char_p, C.c_uint64, C.c_int, C.c_uint64,
       C.c_uint32, C.POINTER(C.c_uint32), C.c_uint64)
_proto("mf_histogram", C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_uint64, C.c_double, C.c_double, C.c_uint32,
       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p)
_proto("mf_kernel_store", C.c_int, c_ker, c_buf, C.c_uint64, C.c_uint64, c_dbl_p, C.c_uint32, c_buf, C.c_uint64)
_proto("mf_kernel_generate", C.c_int, c_ker, C.POINTER(C.c_uint32), C.c_uint32, C.c_uint64, C.c_uint64, c_dbl_p,
       C.c_uint32, c_buf, C.c_uint64, C.c_uint64)
_proto("mf_kernel_generate_async", C.c_int, c_ker, C.POINTER(C.c_uint32), C.c_uint32, C.c_uint64, C.c_uint64, c_dbl_p,
       C.c_uint32, c_buf, C.c_uint64, C.c_uint64)
_proto("mf_kernel_generate_splitmix_async", C.c_int, c_ker, C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint64, c_dbl_p,
       C.c_uint32, c_buf, C.c_uint64, C.c_uint64)
_proto("mf_eval_expressions", C.c_int, C.c_uint32, c_char_pp, c_dbl_p, C.c_uint32, c_char_pp, c_dbl_p)
_proto("mf_seed_rows", C.c_int, C.c_uint64, C.c_uint32, C.POINTER(C.c_uint32))
_proto("mf_splitmix_seed_rows", C.c_int, C.c_uint64, C.c_uint32, C.POINTER(C.c_uint32))
_proto("mf_spd_solve_batch", C.c_int, C.c_uint32, C.c_uint32, c_dbl_p, c_dbl_p, c_dbl_p, c_dbl_p,
       C.POINTER(C.c_uint8))
_proto("mf_generate_partition", C.c_int, C.c_uint64, C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32))
_proto("mf_lower_source", C.c_int, C.POINTER(KernelDesc), C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t))
_proto("mf_compile_check", C.c_int, C.POINTER(KernelDesc), C.POINTER(C.c_int), C.POINTER(C.c_int))
_proto("mf_kernel_reduce_multi", C.c_int, c_ker, C.c_uint32, C.POINTER(c_buf), C.POINTER(C.c_uint64),
       C.POINTER(C.c_uint64), c_dbl_p, C.c_uint32, c_buf)
_proto("mf_coalescer_create", C.c_int, C.c_int, C.c_uint32, C.c_uint32, C.POINTER(c_coal))
_proto("mf_coalescer_destroy", C.c_int, c_coal)
_proto("mf_context_set_coalescer", C.c_int, c_ctx, c_coal)
_proto("mf_coalesced_submit", C.c_int, c_coal, c_ker, c_buf, C.c_uint64, C.c_uint64, c_dbl_p, C.c_uint32,
       C.POINTER(C.c_uint64))
_proto("mf_coalesced_poll", C.c_int, c_coal, C.c_uint64, c_dbl_p, C.c_int)
_proto("mf_coalescer_stats", C.c_int, c_coal, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint32))


def check(rc: int) -> None:
    if rc != MF_OK:
        raise MFError(rc, lib.mf_last_error().decode(errors="replace"))


def cstrings(items) -> C.Array:
    arr = (C.c_char_p * max(1, len(items)))()
    for i, s in enumerate(items):
        arr[i] = s.encode() if isinstance(s, str) else s
    return arr


def dptr(a) -> c_dbl_p:
    return a.ctypes.data_as(c_dbl_p)


def exported_symbols() -> list[str]:
    """Names of every function the header declares (used by the load test)."""
    return [
        "mf_last_error", "mf_version", "mf_device_count", "mf_device_properties", "mf_context_set_resident",
        "mf_context_resident_stats", "mf_compile_check_resident", "mf_context_create", "mf_context_destroy",
        "mf_context_allocated", "mf_context_synchronize", "mf_buffer_alloc", "mf_buffer_free", "mf_buffer_size",
        "mf_buffer_device_ptr", "mf_buffer_h2d", "mf_buffer_d2h", "mf_buffer_memset", "mf_column_stride",
        "mf_events_upload", "mf_events_download", "mf_events_upload_f64_as", "mf_kernel_build", "mf_kernel_free",
        "mf_kernel_source", "mf_kernel_info", "mf_kernel_reduce", "mf_kernel_reduce_async", "mf_kernel_reduce_many",
        "mf_columns_sum", "mf_columns_sum_noalloc", "mf_context_stream", "mf_kernel_reduce_segments", "mf_kernel_store",
        "mf_kernel_generate", "mf_eval_expressions", "mf_seed_rows", "mf_generate_partition", "mf_lower_source",
        "mf_compile_check", "mf_buffer_mark_modified", "mf_kernel_read_layout", "mf_events_upload_async",
        "mf_buffer_d2h_async", "mf_kernel_store_async", "mf_eval_expressions_batch", "mf_kernel_generate_segments",
        "mf_expr_set_create", "mf_expr_set_eval", "mf_expr_set_free", "mf_kernel_fallback_count",
        "mf_histogram", "mf_events_load_file", "mf_splitmix_seed_rows", "mf_buffer_wrap_host",
        "mf_spd_solve_batch", "mf_kernel_reduce_multi", "mf_coalescer_create", "mf_coalescer_destroy",
        "mf_context_set_coalescer", "mf_coalesced_submit", "mf_coalesced_poll", "mf_coalescer_stats",
        "mf_kernel_generate_async", "mf_kernel_reduce_segments_chunked", "mf_kernel_generate_splitmix_async",
    ]
