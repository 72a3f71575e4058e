"""Python mirror of the reference's compute-backend interface on the CUDA C ABI.

``CUDABackend`` and ``CUDABlock`` carry the method names, argument meaning
and call order of ``morefit::ComputeBackend`` / ``morefit::ComputeBlock``
(reference include/compute.hh:98-149), so a test or driver written against
the reference's block interface reads the same here. Event buffers are
numpy arrays of shape ``(ndims, nevents)`` (the SoA layout of EventVector,
include/eventvector.hh:236-260). Kernels are the reference's
``ComputeGraphNode::get_kernel()`` strings.

Every call goes through ``libmorefit_cuda.so``; a failing call raises
``MFError`` instead of the reference's ``assert(0)``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _lib as L


class CUDABackend:
    """One device, one stream, an HBM budget (ComputeBackend, compute.hh:98-107)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, resident_idle_us: int = 2000):
        """``resident_idle_us``: synchronous evaluations of the two most used
        kernels are served by a resident grid that leaves after this long
        without requests (``set_resident``); 0 launches per evaluation."""
        h = L.c_ctx()
        L.check(L.lib.mf_context_create(device, hbm_budget_bytes, C.byref(h)))
        self._h = h
        self.device = device
        if resident_idle_us:
            L.lib.mf_context_set_resident(h, int(resident_idle_us))  # unsupported: launches as usual

    def required_padding(self) -> int:
        # The device layout pads each column internally; host EventVectors
        # stay unpadded (fitter.hh:685-698 then leaves the data alone).
        return 0

    @property
    def handle(self):
        return self._h

    def allocated(self) -> int:
        v = C.c_uint64()
        L.check(L.lib.mf_context_allocated(self._h, C.byref(v)))
        return v.value

    def properties(self) -> dict:
        """Name, SM count and compute capability of this backend's device."""
        name = C.create_string_buffer(256)
        sms, ma, mi = C.c_int(), C.c_int(), C.c_int()
        L.check(L.lib.mf_device_properties(self.device, name, 256, C.byref(sms), C.byref(ma), C.byref(mi)))
        return {"name": name.value.decode(), "sms": sms.value, "cc": (ma.value, mi.value)}

    def synchronize(self) -> None:
        L.check(L.lib.mf_context_synchronize(self._h))

    def set_coalescer(self, coalescer: "Coalescer | None") -> None:
        """Routes this context's synchronous evaluations through `coalescer`
        (None detaches): concurrent fitters in other threads share its launches."""
        L.check(L.lib.mf_context_set_coalescer(self._h, coalescer.handle if coalescer else None))
        self._coalescer = coalescer

    def set_resident(self, idle_us: int) -> None:
        """Serve this context's synchronous evaluations of its most used
        REDUCE kernels from a resident grid (mf_context_set_resident) that
        leaves after ``idle_us`` without requests; 0 turns it off."""
        L.check(L.lib.mf_context_set_resident(self._h, int(idle_us)))

    def resident_stats(self) -> dict:
        st, grids, served, blocks = C.c_int(), C.c_uint64(), C.c_uint64(), C.c_int()
        L.check(L.lib.mf_context_resident_stats(self._h, C.byref(st), C.byref(grids), C.byref(served),
                                                C.byref(blocks)))
        return {"state": st.value, "grids": grids.value, "served": served.value, "blocks": blocks.value}

    def close(self) -> None:
        if getattr(self, "_h", None):
            if getattr(self, "_coalescer", None) is not None:
                L.lib.mf_context_set_coalescer(self._h, None)
                self._coalescer = None
            L.lib.mf_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Coalescer:
    """Gathers the synchronous evaluations of several contexts (one per host
    thread, each running its own fit) into shared launches (mf_coalescer_*)."""

    def __init__(self, device: int = 0, max_batch: int = 0, window_us: int = 30):
        h = L.c_coal()
        L.check(L.lib.mf_coalescer_create(device, max_batch, window_us, C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def stats(self) -> dict:
        t, e, m = C.c_uint64(), C.c_uint64(), C.c_uint32()
        L.check(L.lib.mf_coalescer_stats(self._h, C.byref(t), C.byref(e), C.byref(m)))
        return {"ticks": t.value, "evaluations": e.value, "max_batch": m.value}

    def close(self) -> None:
        if getattr(self, "_h", None):
            L.check(L.lib.mf_coalescer_destroy(self._h))
            self._h = None


class DeviceColumns:
    """A device SoA event block: ``ncols`` columns of ``n`` events, padded stride."""

    def __init__(self, backend: CUDABackend, elem: int):
        self.backend = backend
        self.elem = elem
        self.buf = None
        self._host = None  # the host array of a wrap_host block
        self.ncols = 0
        self.n = 0
        self.stride = 0

    @property
    def itemsize(self) -> int:
        return 4 if self.elem == L.MF_F32 else 8

    def ensure(self, ncols: int, n: int) -> None:
        stride = int(L.lib.mf_column_stride(n))
        need = max(1, ncols) * stride * self.itemsize
        # a block over host memory (wrap_host) is never an upload target
        if self.buf is None or self._host is not None or L.lib.mf_buffer_size(self.buf) < need:
            self.free()
            self._host = None
            b = L.c_buf()
            L.check(L.lib.mf_buffer_alloc(self.backend.handle, need, C.byref(b)))
            self.buf = b
        self.ncols, self.n, self.stride = ncols, n, stride

    def upload(self, events: np.ndarray) -> None:
        ev = np.ascontiguousarray(events)
        if ev.ndim == 1:
            ev = ev[None, :]
        ncols, n = ev.shape
        self.ensure(ncols, n)
        if ev.dtype == np.float64 and self.elem == L.MF_F32:
            L.check(L.lib.mf_events_upload_f64_as(self.buf, L.MF_F32, L.dptr(ev), ncols, n, n, self.stride))
            return
        want = np.float32 if self.elem == L.MF_F32 else np.float64
        ev = np.ascontiguousarray(ev, dtype=want)
        L.check(L.lib.mf_events_upload(self.buf, self.elem, ev.ctypes.data, ncols, n, n, self.stride))

    @classmethod
    def wrap_host(cls, backend: CUDABackend, events: np.ndarray) -> "DeviceColumns":
        """A block over a host SoA array (ncols, n) that kernels read in place
        over the host link (mf_buffer_wrap_host); column stride n. The array
        is kept alive by the block."""
        ev = events if events.ndim == 2 else events[None, :]
        if not ev.flags.c_contiguous or ev.dtype not in (np.float64, np.float32):
            raise ValueError("wrap_host needs a C-contiguous FP64 or FP32 array")
        cols = cls(backend, L.MF_F64 if ev.dtype == np.float64 else L.MF_F32)
        b = L.c_buf()
        L.check(L.lib.mf_buffer_wrap_host(backend.handle, ev.ctypes.data, ev.nbytes, C.byref(b)))
        cols.buf, cols.ncols, cols.n, cols.stride = b, ev.shape[0], ev.shape[1], ev.shape[1]
        cols._host = ev
        return cols

    def download(self) -> np.ndarray:
        out = np.empty((self.ncols, self.n), dtype=np.float32 if self.elem == L.MF_F32 else np.float64)
        L.check(L.lib.mf_events_download(self.buf, self.elem, out.ctypes.data, self.ncols, self.n, self.n,
                                         self.stride))
        return out

    def free(self) -> None:
        if self.buf is not None:
            L.lib.mf_buffer_free(self.buf)
            self.buf = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


@dataclass
class Kernel:
    handle: object
    kind: int
    nout: int
    nparams: int

    def source(self) -> str:
        need = C.c_size_t()
        L.check(L.lib.mf_kernel_source(self.handle, None, 0, C.byref(need)))
        buf = C.create_string_buffer(need.value)
        L.check(L.lib.mf_kernel_source(self.handle, buf, need.value, None))
        return buf.value.decode()

    def info(self) -> dict:
        r, s, b, v = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        L.check(L.lib.mf_kernel_info(self.handle, C.byref(r), C.byref(s), C.byref(b), C.byref(v)))
        return {"registers": r.value, "spill_bytes": s.value, "block": b.value, "vec": v.value}

    def read_layout(self) -> dict:
        """Columns and bytes per event the event loop reads (prepared or source columns)."""
        c, b, sc = C.c_uint32(), C.c_uint32(), C.c_uint32()
        L.check(L.lib.mf_kernel_read_layout(self.handle, C.byref(c), C.byref(b), C.byref(sc)))
        return {"columns": c.value, "bytes_per_event": b.value, "source_columns": sc.value}

    def fallback_count(self) -> int:
        """Reductions evaluated again in native FP64 after a non-finite double-float sum."""
        v = C.c_uint64()
        L.check(L.lib.mf_kernel_fallback_count(self.handle, C.byref(v)))
        return v.value


def make_desc(name: str, kind: int, elem: int, inputs: Sequence[str], params: Sequence[str],
              exprs: Sequence[str], gen=None, native_f64: bool = False, vec: int = 0, block: int = 0,
              f32_arith: bool = False, pipeline: bool = False, stages: int = 0, param_defs=None):
    keep = {"inputs": L.cstrings(list(inputs)), "params": L.cstrings(list(params)),
            "exprs": L.cstrings(list(exprs)), "name": name.encode()}
    d = L.KernelDesc()
    d.name = keep["name"]
    d.kind = kind
    d.elem_type = elem
    d.n_inputs = len(inputs)
    d.input_names = C.cast(keep["inputs"], L.c_char_pp)
    d.n_params = len(params)
    d.param_names = C.cast(keep["params"], L.c_char_pp)
    d.n_outputs = len(exprs)
    d.exprs = C.cast(keep["exprs"], L.c_char_pp)
    d.flags = ((L.MF_FLAG_NATIVE_F64 if native_f64 else 0) | (L.MF_FLAG_F32_ARITH if f32_arith else 0)
               | (L.MF_FLAG_BULK_PIPELINE if pipeline else 0))
    d.vec = vec
    d.block = block
    d.stages = stages
    if param_defs is not None:
        keep["defs"] = (C.c_char_p * len(params))(*[(x or "").encode() if x else None for x in param_defs])
        d.param_defs = C.cast(keep["defs"], L.c_char_pp)
    if gen is not None:
        dims, lo, hi, maxprob = gen
        keep["gd"] = L.cstrings(list(dims))
        keep["lo"] = np.ascontiguousarray(lo, dtype=np.float64)
        keep["hi"] = np.ascontiguousarray(hi, dtype=np.float64)
        d.n_gen_dims = len(dims)
        d.gen_dim_names = C.cast(keep["gd"], L.c_char_pp)
        d.gen_lo = L.dptr(keep["lo"])
        d.gen_hi = L.dptr(keep["hi"])
        d.maxprob = float(maxprob)
    return d, keep


def build_kernel(backend: CUDABackend, name: str, kind: int, elem: int, inputs, params, exprs, gen=None,
                 native_f64: bool = False, vec: int = 0, block: int = 0, f32_arith: bool = False,
                 pipeline: bool = False, stages: int = 0, param_defs=None) -> Kernel:
    d, keep = make_desc(name, kind, elem, inputs, params, exprs, gen, native_f64, vec, block, f32_arith, pipeline, stages,
                        param_defs)
    h = L.c_ker()
    L.check(L.lib.mf_kernel_build(backend.handle, C.byref(d), C.byref(h)))
    del keep
    return Kernel(h, kind, len(exprs), len(params))


def lower_source(name: str, kind: int, elem: int, inputs, params, exprs, gen=None, native_f64: bool = False,
                 vec: int = 0, block: int = 0, f32_arith: bool = False, pipeline: bool = False, stages: int = 0,
                 param_defs=None) -> str:
    """CUDA C the library generates for these expressions (no GPU needed)."""
    d, keep = make_desc(name, kind, elem, inputs, params, exprs, gen, native_f64, vec, block, f32_arith, pipeline, stages,
                        param_defs)
    need = C.c_size_t()
    L.check(L.lib.mf_lower_source(C.byref(d), None, 0, C.byref(need)))
    buf = C.create_string_buffer(need.value)
    L.check(L.lib.mf_lower_source(C.byref(d), buf, need.value, None))
    return buf.value.decode()


def compile_check(name: str, kind: int, elem: int, inputs, params, exprs, gen=None, native_f64: bool = False,
                  vec: int = 0, block: int = 0, f32_arith: bool = False, pipeline: bool = False, stages: int = 0,
                  param_defs=None) -> dict:
    """NVRTC-compiles the lowered kernel for sm_103a without a GPU."""
    d, keep = make_desc(name, kind, elem, inputs, params, exprs, gen, native_f64, vec, block, f32_arith, pipeline, stages,
                        param_defs)
    r, s = C.c_int(), C.c_int()
    L.check(L.lib.mf_compile_check(C.byref(d), C.byref(r), C.byref(s)))
    return {"registers": r.value, "spill_bytes": s.value}


def compile_check_resident(kernels, elem: int, native_f64: bool = False, f32_arith: bool = False) -> dict:
    """NVRTC-compiles the resident module of one or two REDUCE kernels, each
    given as (name, inputs, params, exprs), without a GPU: registers, spilled
    bytes and the module's CUDA C."""
    descs, keep = [], []
    for name, inputs, params, exprs in kernels:
        d, k = make_desc(name, L.MF_KERNEL_REDUCE, elem, inputs, params, exprs, None, native_f64, 0, 0, f32_arith,
                         False, 0, None)
        descs.append(d)
        keep.append(k)
    arr = (C.c_void_p * len(descs))(*[C.addressof(d) for d in descs])
    r, s = C.c_int(), C.c_int()
    buf = C.create_string_buffer(1 << 22)
    L.check(L.lib.mf_compile_check_resident(arr, len(descs), C.byref(r), C.byref(s), buf, len(buf)))
    return {"registers": r.value, "spill_bytes": s.value, "source": buf.value.decode()}


def eval_expressions(names: Sequence[str], values: Sequence[float], exprs: Sequence[str]) -> np.ndarray:
    """Host evaluation of parameter-only expressions (ComputeGraphNode::eval)."""
    v = np.ascontiguousarray(values, dtype=np.float64)
    out = np.zeros(max(1, len(exprs)))
    L.check(L.lib.mf_eval_expressions(len(names), C.cast(L.cstrings(list(names)), L.c_char_pp), L.dptr(v),
                                      len(exprs), C.cast(L.cstrings(list(exprs)), L.c_char_pp), L.dptr(out)))
    return out[: len(exprs)]


def eval_expressions_batch(names: Sequence[str], rows: np.ndarray, exprs: Sequence[str]) -> np.ndarray:
    """eval_expressions for every row of ``rows`` (shape (n_rows, len(names)))."""
    v = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, len(names))
    out = np.zeros((v.shape[0], max(1, len(exprs))))
    L.check(L.lib.mf_eval_expressions_batch(len(names), C.cast(L.cstrings(list(names)), L.c_char_pp), v.shape[0],
                                            L.dptr(v), len(exprs), C.cast(L.cstrings(list(exprs)), L.c_char_pp),
                                            L.dptr(out)))
    return out[:, : len(exprs)]


class ExpressionSet:
    """Parameter-only expressions parsed once (mf_expr_set); ``eval(rows)``
    evaluates them for every row of parameter values."""

    def __init__(self, names: Sequence[str], exprs: Sequence[str]):
        self.n_names, self.n_exprs = len(names), len(exprs)
        self.handle = C.c_void_p()
        L.check(L.lib.mf_expr_set_create(len(names), C.cast(L.cstrings(list(names)), L.c_char_pp), len(exprs),
                                         C.cast(L.cstrings(list(exprs)), L.c_char_pp), C.byref(self.handle)))

    def eval(self, rows) -> np.ndarray:
        v = np.ascontiguousarray(rows, dtype=np.float64).reshape(-1, self.n_names)
        out = np.zeros((v.shape[0], self.n_exprs))
        if self.n_exprs:
            L.check(L.lib.mf_expr_set_eval(self.handle, v.shape[0], L.dptr(v), L.dptr(out)))
        return out

    def __del__(self):
        if getattr(self, "handle", None):
            L.lib.mf_expr_set_free(self.handle)
            self.handle = None


class CUDABlock:
    """ComputeBlock<kernelT, evalT> over the CUDA C ABI (compute.hh:110-149).

    ``kernelT`` is ``np.float64`` (plain FP64) or ``np.float32`` (mixed
    precision: FP32 storage and per-event arithmetic, FP64 sums).
    """

    def __init__(self, backend: CUDABackend, kernelT=np.float64, native_f64: bool = False, vec: int = 0,
                 block: int = 0, f32_arith: bool = False, pipeline: bool = False, stages: int = 0):
        self.backend = backend
        self.native_f64 = native_f64
        self.f32_arith = f32_arith
        self.pipeline = pipeline
        self.shape = (vec, block, stages)
        # FP32 arithmetic over FP64 columns keeps FP64 storage
        self.elem = L.MF_F32 if (np.dtype(kernelT) == np.float32 and not f32_arith) else L.MF_F64
        self.kernelT = np.dtype(kernelT)
        self.input = DeviceColumns(backend, self.elem)
        self.output = DeviceColumns(backend, self.elem)
        self.params = np.zeros(0)
        self.nevents = 0
        self.kernel: Kernel | None = None
        self.kahan = False
        self.nout = 0
        self._sums = np.zeros(0)
        self._seeds = None
        self._gen = None

    # --- buffers (compute.hh:114-128) ---
    def SetupInputBuffer(self, arg, use_data_in: bool = False) -> bool:
        if isinstance(arg, CUDABlock):  # chained: share the other block's device columns
            self.input = arg.input if use_data_in else arg.output
        return True

    def SetupSeedBuffer(self, nbytes: int) -> bool:
        return True

    def SetupParameterBuffer(self, nbytes: int) -> bool:
        return True

    def SetupOutputBuffer(self, nbytes: int) -> bool:
        return True

    def SetupKahanBuffer(self, nbytes: int) -> bool:
        self._sums = np.zeros(nbytes // 8)
        return True

    def SetNevents(self, nevents: int, nevents_padded: int = -1) -> bool:
        self.nevents = int(nevents)
        return True

    # --- copies (compute.hh:130-138) ---
    def CopyToInputBuffer(self, events: np.ndarray) -> bool:
        self.input.upload(events)
        self.nevents = self.input.n
        return True

    def CopyToInputBufferAsync(self, events: np.ndarray) -> bool:
        """Stream-ordered upload: `events` (contiguous, page-locked for overlap) must
        stay valid and unchanged until Finish()."""
        ev = events if events.ndim == 2 else events[None, :]
        if not ev.flags.c_contiguous or ev.dtype != (np.float32 if self.elem == L.MF_F32 else np.float64):
            raise ValueError("asynchronous upload needs a contiguous array of the block's element type")
        ncols, n = ev.shape
        self.input.ensure(ncols, n)
        L.check(L.lib.mf_events_upload_async(self.input.buf, self.elem, ev.ctypes.data, ncols, n, n,
                                             self.input.stride))
        self.nevents = n
        return True

    def SubmitKernelAsync(self, out=None, out_index: int = 0) -> bool:
        """SubmitKernel without waiting: STORE kernels write the output columns;
        REDUCE kernels write their sums to row `out_index` of device buffer `out`."""
        k = self.kernel
        p = self.params if self.params.size else np.zeros(1)
        if k.kind == L.MF_KERNEL_STORE:
            self.output.ensure(k.nout, self.nevents)
            L.check(L.lib.mf_kernel_store_async(k.handle, self.input.buf, self.input.stride, self.nevents,
                                                L.dptr(p), k.nparams, self.output.buf, self.output.stride))
        elif k.kind == L.MF_KERNEL_REDUCE:
            L.check(L.lib.mf_kernel_reduce_async(k.handle, self.input.buf, self.input.stride, self.nevents,
                                                 L.dptr(p), k.nparams, out, out_index))
        else:  # generate: out = events per generator thread (None: spread over the seed rows)
            nseeds = self._seeds.shape[-1] if self._seeds.ndim == 2 else self._seeds.size // 4
            per = out if out else -(-self.nevents // nseeds)
            self.output.ensure(self._gen, self.nevents)
            L.check(L.lib.mf_kernel_generate_async(k.handle, self._seeds.ctypes.data_as(C.POINTER(C.c_uint32)),
                                                   nseeds, self.nevents, per, L.dptr(p), k.nparams, self.output.buf,
                                                   self.output.stride, 10000 * per))
        return True

    def SubmitGenerateSplitmixAsync(self, seed: int, nstreams: int, nper: int) -> bool:
        """Generation without a seed table: `nstreams` streams seeded on the
        device as splitmix_seed_rows(nstreams, seed) seeds them (the same
        events), enqueued without a host wait (mf_kernel_generate_splitmix_async)."""
        k = self.kernel
        p = self.params if self.params.size else np.zeros(1)
        self.output.ensure(self._gen, self.nevents)
        L.check(L.lib.mf_kernel_generate_splitmix_async(k.handle, int(seed), int(nstreams), self.nevents, int(nper),
                                                        L.dptr(p), k.nparams, self.output.buf, self.output.stride,
                                                        10000 * int(nper)))
        return True

    def CopyToSeedBuffer(self, seeds: np.ndarray) -> bool:
        self._seeds = np.ascontiguousarray(seeds, dtype=np.uint32)
        return True

    def CopyToParameterBuffer(self, params) -> bool:
        self.params = np.ascontiguousarray(params, dtype=np.float64)
        return True

    def CopyFromOutputBuffer(self) -> np.ndarray:
        return self.output.download()

    def CopyFromKahanBuffer(self) -> np.ndarray:
        return self._sums.copy()

    # --- kernels (compute.hh:140-148) ---
    def MakeComputeKernel(self, name: str, nevents: int, input_signature: Sequence[str],
                          output_signature: Sequence[str], params: Sequence[str], graphs: Sequence[str],
                          kahan_summation: bool = False, param_defs=None) -> bool:
        """``param_defs``: optional, per parameter "" or its defining expression
        (the fitter's hoisted parameter buffers); helps the lowering fold columns."""
        if len(output_signature) != len(graphs):
            raise ValueError("output_signature and graphs differ in length (compute_opencl.hh:707)")
        self.kahan = bool(kahan_summation)
        self.nout = len(graphs)
        kind = L.MF_KERNEL_REDUCE if self.kahan else L.MF_KERNEL_STORE
        self.kernel = build_kernel(self.backend, name, kind, self.elem, input_signature, params, graphs,
                                   native_f64=self.native_f64, vec=self.shape[0], block=self.shape[1],
                                   f32_arith=self.f32_arith and kind == L.MF_KERNEL_REDUCE, pipeline=self.pipeline,
                                   stages=self.shape[2], param_defs=param_defs)
        self._sums = np.zeros(self.nout)
        self.nevents = int(nevents)
        return True

    def MakeGenerateKernel(self, name: str, nevents: int, input_signature, output_signature: Sequence[str],
                           params, graphs: Sequence[str], maxprob: float = 1.0, ranges=None) -> bool:
        dims = [d[0] if isinstance(d, tuple) else d for d in output_signature]
        lo = [r[0] for r in ranges]
        hi = [r[1] for r in ranges]
        self.kernel = build_kernel(self.backend, name, L.MF_KERNEL_GENERATE, self.elem, [], params, graphs,
                                   gen=(dims, lo, hi, maxprob))
        self._gen = len(dims)
        self.nevents = int(nevents)
        return True

    def SubmitKernel(self, nper: int | None = None, max_tries: int | None = None) -> bool:
        k = self.kernel
        if k is None:
            raise RuntimeError("SubmitKernel before MakeComputeKernel")
        p = self.params if self.params.size else np.zeros(1)
        if k.kind == L.MF_KERNEL_REDUCE:
            sums = np.zeros(k.nout)
            L.check(L.lib.mf_kernel_reduce(k.handle, self.input.buf, self.input.stride, self.nevents, L.dptr(p),
                                           k.nparams, L.dptr(sums)))
            self._sums = sums
        elif k.kind == L.MF_KERNEL_STORE:
            self.output.ensure(k.nout, self.nevents)
            L.check(L.lib.mf_kernel_store(k.handle, self.input.buf, self.input.stride, self.nevents, L.dptr(p),
                                          k.nparams, self.output.buf, self.output.stride))
        else:
            nseeds = self._seeds.shape[-1] if self._seeds.ndim == 2 else self._seeds.size // 4
            per = nper if nper else -(-self.nevents // nseeds)
            if max_tries is None:  # every thread gives up after 10^4 proposals per event it owns
                max_tries = 10000 * per
            self.output.ensure(self._gen, self.nevents)
            L.check(L.lib.mf_kernel_generate(k.handle, self._seeds.ctypes.data_as(C.POINTER(C.c_uint32)), nseeds,
                                             self.nevents, per, L.dptr(p), k.nparams, self.output.buf,
                                             self.output.stride, max_tries))
        return True

    def Finish(self) -> bool:
        self.backend.synchronize()
        return True

    def ProvidesKahan(self) -> bool:
        return True

    # --- batched ragged segments (toy studies) ---
    def SubmitSegments(self, seg_begin, seg_count, params_rows, events_per_block: int = 0) -> np.ndarray:
        """Sums of every segment [seg_begin[s], seg_begin[s] + seg_count[s]) at
        its own parameter row: one block per segment, or (``events_per_block``
        > 0) runs of that many events of each segment, one block each."""
        k = self.kernel
        b = np.ascontiguousarray(seg_begin, dtype=np.uint64)
        c = np.ascontiguousarray(seg_count, dtype=np.uint32)
        pr = np.ascontiguousarray(params_rows, dtype=np.float64).reshape(len(b), -1)
        out = np.zeros((len(b), k.nout))
        pb, pc = b.ctypes.data_as(C.POINTER(C.c_uint64)), c.ctypes.data_as(C.POINTER(C.c_uint32))
        if events_per_block > 0:
            L.check(L.lib.mf_kernel_reduce_segments_chunked(k.handle, self.input.buf, self.input.stride, len(b), pb,
                                                            pc, L.dptr(pr), k.nparams, events_per_block,
                                                            L.dptr(out)))
        else:
            L.check(L.lib.mf_kernel_reduce_segments(k.handle, self.input.buf, self.input.stride, len(b), pb, pc,
                                                    L.dptr(pr), k.nparams, L.dptr(out)))
        return out
