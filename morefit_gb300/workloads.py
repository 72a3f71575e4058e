"""Likelihood evaluation on the CUDA backend for a lowered MoreFit model.

A model spec (``morefit_gb300/specs/<name>.json``) holds exactly what the
reference's ``fitter::make_kernels`` hands its compute backend
(include/fitter.hh:321-658): the precompute kernel (event-only hoisted
columns), the lh / lh+grad / Hessian kernels as get_kernel() strings, and the
parameter-buffer expressions evaluated on the host before every launch.

``Likelihood`` restates the fitter's evaluation calls on top of
``CUDABlock`` with the same call sequence and the same conventions:
``likelihood()`` returns -2 sum log p (fitter.hh:1152-1220),
``likelihood_and_gradient()`` returns (-2 sum log p, -2 sum dlogp/dtheta)
(fitter.hh:1054-1151) and ``hessian()`` returns the matrix of -2 sum
d2logp/dtheta_i dtheta_j (fitter.hh:1221-1326). The event block is uploaded
once (fitter.hh:704-757) and every evaluation moves only the parameter
vector in and the sums out.

Weighted data (a spec with a ``weight`` column): the reference multiplies
log p by the weight column (fitter.hh:337-338), builds the Fisher kernel
d(w log p)/dtheta_i * d(w log p)/dtheta_j (fitter.hh:471-523), and corrects
the covariance to -2 H^-1 F H^-1 (fitter.hh:894-943). ``fisher()`` and
``corrected_covariance()`` restate those two steps.
"""
from __future__ import annotations

import json
import re
from pathlib import Path

import numpy as np

import ctypes as C

from . import _lib as L
from .backend import CUDABackend, CUDABlock, DeviceColumns, ExpressionSet

DEFAULT_SEED = 229387429
MAX_GENERATOR_WORKITEMS = 8192  # compute_options::opencl_max_generator_workitems (compute.hh:59)

SPEC_DIR = Path(__file__).resolve().parent / "specs"


def load_spec(name: str) -> dict:
    return json.loads((SPEC_DIR / f"{name}.json").read_text())


def weighted_covariance(hessian: np.ndarray, fisher: np.ndarray) -> np.ndarray:
    """-2 H^-1 F H^-1 from H = -2 sum d2(w log p) and F = -2 sum d(w log p) d(w log p)
    (fitter.hh:931-933): the sandwich (sum w d2 log p)^-1 (sum w^2 d log p d log p)
    (sum w d2 log p)^-1 in the fitter's -2 ln L convention."""
    hinv = np.linalg.inv(np.asarray(hessian, dtype=np.float64))
    return -2.0 * hinv @ np.asarray(fisher, dtype=np.float64) @ hinv


class Likelihood:
    """NLL, gradient and Hessian of one dataset, device resident."""

    def __init__(self, backend: CUDABackend, spec: dict, kernelT=np.float64, native_f64: bool = False, vec: int = 0,
                 block: int = 0, pipeline: bool = False, stages: int = 0):
        self.backend = backend
        self.spec = spec
        self.kernelT = np.dtype(kernelT)
        self.params = list(spec["parameters"])
        ks = {k["name"]: k for k in spec["kernels"]}
        self.kspec = ks
        self.has_precompute = "precompute_kernel" in ks
        self.buffers = {"lh_kernel": spec["lh_buffers"], "lh_grad_kernel": spec["grad_buffers"],
                        "lh_hessian_kernel": spec["hessian_buffers"],
                        "lh_fisher_kernel": spec.get("fisher_buffers", [])}
        self.weight = spec.get("weight")
        # Blocks as the fitter wires them (fitter.hh:525-657, 704-757). In
        # mixed precision the hoisted basis columns are stored in FP32; a model
        # without them reads its raw observables, which keep FP64 storage with
        # FP32 arithmetic (MF_FLAG_F32_ARITH).
        mixed_raw = self.kernelT == np.float32 and not self.has_precompute
        # The precompute runs in double-float (FP32 pipe) unless native FP64 is asked for.
        self.pre = CUDABlock(backend, np.float64 if mixed_raw else kernelT, native_f64=native_f64)
        self.blocks = {}
        self._block_args = dict(native_f64=native_f64, vec=vec, block=block, f32_arith=mixed_raw, pipeline=pipeline,
                                stages=stages)
        for name in ("lh_kernel", "lh_grad_kernel", "lh_hessian_kernel", "lh_fisher_kernel"):
            if name not in ks:
                continue
            b = CUDABlock(backend, kernelT, **self._block_args)
            if self.has_precompute:
                b.SetupInputBuffer(self.pre, False)
            else:
                b.SetupInputBuffer(self.pre, True)
            k = ks[name]
            defs = dict(self.buffers[name])
            b.MakeComputeKernel(name, 0, k["inputs"], [f"r{i}" for i in range(len(k["exprs"]))], k["params"],
                                k["exprs"], True, param_defs=[defs.get(p, "") for p in k["params"]])
            self.blocks[name] = b
        if self.has_precompute:
            k = ks["precompute_kernel"]
            self.pre.MakeComputeKernel("precompute_kernel", 0, k["inputs"], k["outputs"], [], k["exprs"], False)
        self.nevents = 0

    def set_data(self, events: np.ndarray) -> None:
        """Uploads the raw event block (ndims, n) and runs the precompute kernel."""
        ev = np.asarray(events)
        if ev.ndim == 1:
            ev = ev[None, :]
        self.pre.CopyToInputBuffer(ev)
        self.nevents = ev.shape[1]
        if self.has_precompute:
            self.pre.SetNevents(self.nevents)
            self.pre.SubmitKernel()
        for b in self.blocks.values():
            b.SetNevents(self.nevents)

    def set_data_async(self, events: np.ndarray) -> None:
        """set_data without host waits: upload and precompute are enqueued on the
        backend's stream; `events` (contiguous FP64, page-locked for overlap) must
        stay valid until the backend is synchronized."""
        ev = events if events.ndim == 2 else events[None, :]
        self.pre.CopyToInputBufferAsync(ev)
        self.nevents = ev.shape[1]
        if self.has_precompute:
            self.pre.SetNevents(self.nevents)
            self.pre.SubmitKernelAsync()
        for b in self.blocks.values():
            b.SetNevents(self.nevents)

    def set_data_mapped(self, events: np.ndarray) -> None:
        """set_data without a copy to HBM: the precompute kernel (or, without
        one, the column preparation) reads `events` (contiguous FP64,
        page-locked) in place over the host link while it computes. Enqueued
        without host waits; `events` must stay valid and unchanged until the
        backend is synchronized."""
        ev = events if events.ndim == 2 else events[None, :]
        cached = self.__dict__.get("_mapped")
        if cached is None or cached._host is not ev:
            cached = DeviceColumns.wrap_host(self.backend, ev)
            self._mapped = cached
        else:
            L.check(L.lib.mf_buffer_mark_modified(cached.buf))
        self.pre.input = cached
        self.nevents = ev.shape[1]
        if self.has_precompute:
            self.pre.SetNevents(self.nevents)
            self.pre.SubmitKernelAsync()
        else:
            for b in self.blocks.values():
                b.SetupInputBuffer(self.pre, True)
        for b in self.blocks.values():
            b.SetNevents(self.nevents)

    def sums_async(self, kernel: str, theta, out, out_index: int = 0) -> None:
        """Enqueues one evaluation whose sums land in row `out_index` of device buffer `out`."""
        b = self.blocks[kernel]
        b.CopyToParameterBuffer(self.param_vector(kernel, theta))
        b.SubmitKernelAsync(out, out_index)

    def set_device_data(self, cols: DeviceColumns) -> None:
        """Uses an event block already on the device (e.g. from generate_events)."""
        if cols.elem != self.pre.elem:
            self.set_data(cols.download())
            return
        self.pre.input = cols
        self.nevents = cols.n
        if self.has_precompute:
            self.pre.SetNevents(self.nevents)
            self.pre.SubmitKernel()
        else:
            for b in self.blocks.values():
                b.SetupInputBuffer(self.pre, True)
        for b in self.blocks.values():
            b.SetNevents(self.nevents)

    def input_block(self, kernel: str = "lh_grad_kernel") -> DeviceColumns:
        return self.blocks[kernel].input

    def _exprs(self, kernel: str) -> ExpressionSet:
        cache = self.__dict__.setdefault("_expr_sets", {})
        if kernel not in cache:
            cache[kernel] = ExpressionSet(self.params, [e for _, e in self.buffers[kernel]])
        return cache[kernel]

    def param_vector(self, kernel: str, theta) -> np.ndarray:
        """[floating values..., parameter buffers...] as the fitter builds it (fitter.hh:1059-1072)."""
        return self.param_rows(kernel, np.asarray(theta, dtype=np.float64)[None, :])[0]

    def param_rows(self, kernel: str, thetas) -> np.ndarray:
        """param_vector for every row of ``thetas`` (n, n_floating)."""
        th = np.atleast_2d(np.asarray(thetas, dtype=np.float64))
        if not self.buffers[kernel]:
            return th.copy()
        return np.concatenate([th, self._exprs(kernel).eval(th)], axis=1)

    HESSIAN_PART_OUTPUTS = 36  # the K*mumu P-wave Hessian's size, which keeps its accumulators in registers

    def kernel_parts(self, kernel: str) -> list:
        """Kernels whose outputs, concatenated, are ``kernel``'s: the kernel
        itself, or for a Hessian kernel that spills more than
        COMBINED_MAX_SPILL bytes of registers, equal slices of its outputs of
        at most HESSIAN_PART_OUTPUTS each, one kernel per slice, built on
        first use (each part repeats the per-event work the slice needs and
        reads the dataset again). The lowering keeps many-output kernels
        such as the S+P-wave Hessian (105 outputs) from spilling (partials
        beyond MF_NREG in shared memory), so they stay one kernel."""
        parts = self.__dict__.setdefault("_parts", {})
        if kernel in parts:
            return parts[kernel]
        res = [kernel]
        k, b = self.kspec.get(kernel), self.blocks.get(kernel)
        if kernel == "lh_hessian_kernel" and b is not None and len(k["exprs"]) > self.HESSIAN_PART_OUTPUTS \
                and b.kernel.info()["spill_bytes"] > self.COMBINED_MAX_SPILL:
            exprs = k["exprs"]
            m = -(-len(exprs) // self.HESSIAN_PART_OUTPUTS)
            size = -(-len(exprs) // m)
            defs = dict(self.buffers[kernel])
            res = []
            for i in range(m):
                name = f"{kernel}_part{i}"
                sub = exprs[i * size:(i + 1) * size]
                nb = CUDABlock(self.backend, self.kernelT, **self._block_args)
                nb.SetupInputBuffer(self.pre, not self.has_precompute)
                nb.MakeComputeKernel(name, 0, k["inputs"], [f"r{j}" for j in range(len(sub))], k["params"], sub, True,
                                     param_defs=[defs.get(p, "") for p in k["params"]])
                nb.SetNevents(self.nevents)
                self.buffers[name] = self.buffers[kernel]
                self.blocks[name] = nb
                res.append(name)
        parts[kernel] = res
        return res

    def sums(self, kernel: str, theta=None, param_vector=None) -> np.ndarray:
        parts = self.kernel_parts(kernel)
        if parts != [kernel]:
            return np.concatenate([self.sums(p, theta, param_vector) for p in parts])
        if param_vector is None:
            calls = self.__dict__.setdefault("_sync_calls", {})
            call = calls.get(kernel)
            if call is None:
                call = calls[kernel] = _SyncEvaluation(self, kernel)
            return call(theta)
        b = self.blocks[kernel]
        pv = np.asarray(param_vector, np.float64)
        b.CopyToParameterBuffer(pv)
        b.SubmitKernel()
        return b.CopyFromKahanBuffer()

    def sums_many(self, kernel: str, thetas) -> np.ndarray:
        """The sums at several parameter points (rows of ``thetas``) in one
        batched call (mf_kernel_reduce_many: consecutive evaluations overlap,
        one combine per chunk); each row equals ``sums(kernel, theta)`` bit
        for bit. Returns (npoints, noutputs)."""
        parts = self.kernel_parts(kernel)
        if parts != [kernel]:
            return np.concatenate([self.sums_many(p, thetas) for p in parts], axis=1)
        b = self.blocks[kernel]
        k = b.kernel
        rows = np.ascontiguousarray(self.param_rows(kernel, thetas))
        count = rows.shape[0]
        out = L.c_buf()
        L.check(L.lib.mf_buffer_alloc(self.backend.handle, count * k.nout * 8, C.byref(out)))
        try:
            ins = (L.c_buf * count)(*([b.input.buf] * count))
            strides = np.full(count, b.input.stride, dtype=np.uint64)
            ns = np.full(count, self.nevents, dtype=np.uint64)
            u64p = C.POINTER(C.c_uint64)
            L.check(L.lib.mf_kernel_reduce_many(k.handle, count, ins, strides.ctypes.data_as(u64p),
                                                ns.ctypes.data_as(u64p), L.dptr(rows), rows.shape[1], out))
            res = np.empty((count, k.nout))
            L.check(L.lib.mf_buffer_d2h(out, 0, res.ctypes.data, res.nbytes))
        finally:
            L.lib.mf_buffer_free(out)
        return res

    def likelihood(self, theta) -> float:
        return -2.0 * float(self.sums("lh_kernel", theta)[0])

    def likelihood_and_gradient(self, theta):
        s = self.sums("lh_grad_kernel", theta)
        return -2.0 * float(s[0]), -2.0 * s[1:]

    def _symmetric(self, s: np.ndarray) -> np.ndarray:
        """-2 * the lower-triangle sums (row i, columns j <= i) as a full matrix."""
        npar = len(self.params)
        h = np.zeros((npar, npar))
        idx = 0
        for i in range(npar):
            for j in range(i + 1):
                h[i, j] = h[j, i] = -2.0 * s[idx]
                idx += 1
        return h

    def hessian(self, theta) -> np.ndarray:
        return self._symmetric(self.sums("lh_hessian_kernel", theta))

    COMBINED = "lh_grad_hessian_kernel"
    COMBINED_MAX_SPILL = 64  # bytes per thread (a few values of call frame)

    def combined_kernel(self):
        """Name of the F + gradient + Hessian kernel (the gradient kernel's
        outputs followed by the Hessian kernel's, in one launch that shares
        their common subexpressions; the Hessian's parameter buffers renamed),
        built on first use. None where the model has no Hessian kernel, the
        two kernels read different inputs or parameter buffers, or the
        combined kernel would spill more than COMBINED_MAX_SPILL bytes of
        registers."""
        if "_combined" in self.__dict__:
            return self._combined
        self._combined = None
        ks = self.kspec
        if "lh_grad_kernel" not in ks or "lh_hessian_kernel" not in ks:
            return None
        g, h = ks["lh_grad_kernel"], ks["lh_hessian_kernel"]
        nth = len(self.params)
        gbuf, hbuf = self.buffers["lh_grad_kernel"], self.buffers["lh_hessian_kernel"]
        if g["inputs"] != h["inputs"] or list(g["params"][nth:]) != [n for n, _ in gbuf] \
                or list(h["params"][nth:]) != [n for n, _ in hbuf] or g["params"][:nth] != h["params"][:nth]:
            return None

        def ren(e):
            return re.sub(r"\bmorefit_parambuffer_(\d+)\b", r"mfh_parambuffer_\1", e)
        hb = [(ren(n), ren(e)) for n, e in hbuf]
        params = list(g["params"]) + [n for n, _ in hb]
        exprs = list(g["exprs"]) + [ren(e) for e in h["exprs"]]
        defs = dict(gbuf)
        defs.update(dict(hb))
        b = CUDABlock(self.backend, self.kernelT, **self._block_args)
        b.SetupInputBuffer(self.pre, not self.has_precompute)
        b.MakeComputeKernel(self.COMBINED, 0, g["inputs"], [f"r{i}" for i in range(len(exprs))], params, exprs, True,
                            param_defs=[defs.get(p, "") for p in params])
        if b.kernel.info()["spill_bytes"] > self.COMBINED_MAX_SPILL:
            return None
        b.SetNevents(self.nevents)
        self.buffers[self.COMBINED] = list(gbuf) + hb
        self.blocks[self.COMBINED] = b
        self._combined = self.COMBINED
        return self._combined

    def value_gradient_hessian(self, theta):
        """(-2 ln L, its gradient, its Hessian) at theta: one launch of the
        combined kernel where it exists, else the two kernels."""
        name = self.combined_kernel()
        if name is None:
            f, g = self.likelihood_and_gradient(theta)
            return f, g, self.hessian(theta)
        s = self.sums(name, theta)
        npar = len(self.params)
        return -2.0 * float(s[0]), -2.0 * s[1:1 + npar], self._symmetric(s[1 + npar:])

    def fisher(self, theta) -> np.ndarray:
        """-2 sum d(w log p)/dtheta_i d(w log p)/dtheta_j (fitter.hh:1328-1370)."""
        if "lh_fisher_kernel" not in self.blocks:
            raise ValueError("the model has no Fisher kernel (unweighted data)")
        return self._symmetric(self.sums("lh_fisher_kernel", theta))

    def corrected_covariance(self, theta) -> np.ndarray:
        """Covariance of a weighted fit at theta (fitter.hh:894-943)."""
        return weighted_covariance(self.hessian(theta), self.fisher(theta))

    def fit(self, theta0=None, limits=None, tol: float = 1e-9):
        """Minimises -2 ln L of the whole dataset from theta0 (default: the
        spec's truth) within limits (default: none) by damped Newton steps
        on the analytic gradient and Hessian, the derivative information the
        reference's MIGRAD + HESSE run uses (fitter.hh:659-1000). Errors come
        from 2 H^-1 (errordef 1), or for weighted data from the corrected
        covariance, as the reference reports them (fitter.hh:894-994).
        Returns a FitResult with one row."""
        from .toystudy import fit_segments
        th0 = np.asarray(self.spec["truth"] if theta0 is None else theta0, dtype=np.float64)[None, :]
        lim = limits if limits is not None else [(-np.inf, np.inf)] * len(self.params)
        r = fit_segments(_WholeDataset(self), th0, lim, tol=tol)
        if self.weight is not None:
            r.errors[0] = np.sqrt(np.abs(np.diag(self.corrected_covariance(r.values[0]))))
        return r


class _SyncEvaluation:
    """One synchronous evaluation of a REDUCE kernel at the floating
    parameter values, the fitter's per-call path (fitter.hh:1054-1151) with
    the host work cut to two C calls: the parameter vector [floating
    values..., parameter buffers...] lives in one preallocated array whose
    hoisted buffers mf_expr_set_eval writes in place, and the sums land in a
    second one; both pointers are made once."""

    __slots__ = ("like", "block", "handle", "ntheta", "nparams", "pv", "out", "exprs", "pv_p", "bufs_p", "out_p")

    def __init__(self, like: Likelihood, kernel: str):
        b = like.blocks[kernel]
        k = b.kernel
        self.like, self.block, self.handle = like, b, k.handle
        self.ntheta = len(like.params)
        self.nparams = self.ntheta + len(like.buffers[kernel])
        if self.nparams != k.nparams:
            raise ValueError(f"{kernel}: {k.nparams} kernel parameters, {self.nparams} in the parameter vector")
        self.pv = np.zeros(max(1, self.nparams))
        self.out = np.zeros(k.nout)
        self.exprs = like._exprs(kernel) if self.nparams > self.ntheta else None
        self.pv_p = L.dptr(self.pv)
        self.bufs_p = C.cast(self.pv.ctypes.data + 8 * self.ntheta, L.c_dbl_p)
        self.out_p = L.dptr(self.out)

    def __call__(self, theta) -> np.ndarray:
        self.pv[:self.ntheta] = theta
        if self.exprs is not None:
            L.check(L.lib.mf_expr_set_eval(self.exprs.handle, 1, self.pv_p, self.bufs_p))
        b = self.block
        L.check(L.lib.mf_kernel_reduce(self.handle, b.input.buf, b.input.stride, b.nevents, self.pv_p, self.nparams,
                                       self.out_p))
        return self.out.copy()


class _WholeDataset:
    """The batched-fit interface (value, value_and_gradient, hessian of rows
    of parameters) over one whole dataset through the full-grid kernels."""

    def __init__(self, like: Likelihood):
        self.like = like
        self.params = like.params
        self.evaluations = 0

    def value(self, idx, theta):
        self.evaluations += len(theta)
        return np.array([self.like.likelihood(t) for t in theta])

    def value_and_gradient(self, idx, theta):
        self.evaluations += len(theta)
        fg = [self.like.likelihood_and_gradient(t) for t in theta]
        return np.array([f for f, _ in fg]), np.array([g for _, g in fg])

    def hessian(self, idx, theta):
        self.evaluations += len(theta)
        return np.array([self.like.hessian(t) for t in theta])

    def value_gradient_hessian(self, idx, theta):
        self.evaluations += len(theta)
        fgh = [self.like.value_gradient_hessian(t) for t in theta]
        return (np.array([f for f, _, _ in fgh]), np.array([g for _, g, _ in fgh]),
                np.array([h for _, _, h in fgh]))


def seed_rows(nrows: int, seed: int = DEFAULT_SEED) -> np.ndarray:
    out = np.zeros((4, nrows), dtype=np.uint32)
    L.check(L.lib.mf_seed_rows(seed, nrows, out.ctypes.data_as(C.POINTER(C.c_uint32))))
    return out


def splitmix_seed_rows(nrows: int, seed: int) -> np.ndarray:
    """xoshiro128++ states (SoA [4][nrows]) seeded independently per stream:
    the upper halves of four SplitMix64 outputs from seed * 2^32 + row (for
    generations that need independent streams rather than the reference's
    jump partition, which seed_rows reproduces)."""
    out = np.zeros((4, nrows), dtype=np.uint32)
    L.check(L.lib.mf_splitmix_seed_rows(seed, nrows, out.ctypes.data_as(C.POINTER(C.c_uint32))))
    return out


def generate_partition(n: int, max_workitems: int = MAX_GENERATOR_WORKITEMS):
    nper, nseeds = C.c_uint64(), C.c_uint32()
    L.check(L.lib.mf_generate_partition(n, max_workitems, C.byref(nper), C.byref(nseeds)))
    return nper.value, nseeds.value


def generate_events(backend: CUDABackend, spec: dict, n: int, seed: int = DEFAULT_SEED,
                    max_workitems: int = MAX_GENERATOR_WORKITEMS, kernelT=np.float64) -> DeviceColumns:
    """Seeded accept-reject events on the GPU (generator::generate, generator.hh:71-175).

    Uses the model's generate kernel (the normalised density with the truth
    values substituted, as the reference's generator builds it) and the
    accelerator work partition with ``max_workitems`` generator threads."""
    gk = next(k for k in spec["kernels"] if k.get("generate"))
    blk = CUDABlock(backend, kernelT)
    blk.MakeGenerateKernel(gk["name"], n, [], gk["outputs"], gk["params"], gk["exprs"], gk["maxprob"],
                           ranges=list(zip(gk["lo"], gk["hi"])))
    nper, nseeds = generate_partition(n, max_workitems)
    blk.CopyToSeedBuffer(seed_rows(nseeds, seed))
    blk.SetNevents(n)
    blk.SubmitKernel(nper=nper)
    cols = blk.output
    blk.output = DeviceColumns(backend, blk.elem)  # hand the columns over to the caller
    return cols


def elem_of(kernelT) -> int:
    return L.MF_F32 if np.dtype(kernelT) == np.float32 else L.MF_F64
