"""Serving loop: many fits at once on one GPU, their evaluations coalesced.

Fit requests (a model, an event count, a seed, start values) arrive over
time. Each admitted fit keeps its dataset on the device (generated there and
precomputed once, both enqueued without host waits so that admitting many
requests costs no round trips) and is driven by a host-side minimiser
written as a coroutine that yields evaluation requests, the way the
reference's Minuit2 asks its FCN for -2 ln L, the gradient and, with the
analytic Hessian switched on, the Hessian (include/fitter.hh:113-169). The server runs in ticks: it admits the
requests that have arrived while the HBM budget and the slots allow, takes
the pending evaluation of every active fit, issues one launch per (model,
kernel) over all of them (mf_kernel_reduce_multi: each dataset cut into
segments of 2048 events, one block each), hands each fit its sums and frees
the dataset of every fit that finishes. Requests that arrive while others are
on the GPU join at the next tick (continuous batching). A dataset's sums in
such a launch do not depend on what else shares it, so every fit follows the
same trajectory alone and in the mix.

The minimiser uses the information the reference's fit uses with analytic
derivatives switched on (gradient and Hessian kernels): damped Newton steps
on F = -2 ln L inside the parameter limits until the estimated distance to
the minimum g^T H^-1 g / 2 is below ``edm_tol`` (2e-5: MIGRAD's 0.002 x
tolerance x errordef at tolerance 0.01); errors are sqrt(diag(2 H^-1))
(errordef 1).
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .backend import CUDABackend, CUDABlock, DeviceColumns
from .workloads import Likelihood, load_spec


MODEL_LIMITS = {
    "mass": [(5200.0, 5400.0), (5.0, 50.0), (0.0, 1.0), (-0.01, 0.01)],
    "pwave": [(0.0, 1.0)] + [(-1.0, 1.0)] * 7,
    "spwave": [(0.0, 1.0)] + [(-1.0, 1.0)] * 7 + [(0.0, 1.0)] + [(-1.0, 1.0)] * 5,
}


@dataclass
class FitRequest:
    id: int
    model: str
    nevents: int
    seed: int
    arrival: float = 0.0           # seconds after the stream starts
    start: np.ndarray | None = None


@dataclass
class FitOutcome:
    id: int
    model: str
    nevents: int
    values: np.ndarray
    errors: np.ndarray
    fmin: float
    evaluations: int
    converged: bool
    admitted: float
    finished: float
    latency: float                 # finished - arrival


def newton_fit(theta0, limits, edm_tol: float = 2e-5, max_iter: int = 100, f_noise: float = 0.0,
               max_halvings: int = 30, combined: bool = False):
    """Coroutine minimiser of F = -2 ln L with the analytic Hessian: damped
    Newton steps inside the parameter limits, halved until F does not rise
    by more than its own precision (``f_noise`` relative: a few 1e-9 for FP32
    per-event arithmetic with compensated sums), until the estimated distance
    to the minimum g^T H^-1 g / 2 is below ``edm_tol``. Yields ("grad", theta)
    and ("hess", theta), receives (F, gradient) and the Hessian; with
    ``combined`` it yields ("gh", theta) instead and receives (F, gradient,
    Hessian) from one evaluation, at the start point and at every step trial,
    so an accepted step needs no separate Hessian request. Returns (theta,
    errors, F, converged, evaluations), errors sqrt(diag(2 H^-1))."""
    lo = np.array([a for a, _ in limits])
    hi = np.array([b for _, b in limits])
    x = np.clip(np.array(theta0, dtype=np.float64), lo, hi)
    n_eval = 0
    converged = False
    h = None
    if combined:
        f, g, h = yield ("gh", x)
    else:
        f, g = yield ("grad", x)
    n_eval += 1
    for _ in range(max_iter):
        if not combined:
            h = yield ("hess", x)
            n_eval += 1
        try:
            p = -np.linalg.solve(h, g)
        except np.linalg.LinAlgError:
            p = -np.linalg.lstsq(h, g, rcond=None)[0]
        edm = -0.5 * g @ p
        if not np.isfinite(edm) or edm <= 0:  # not positive definite here: scaled gradient step
            p = -g / np.maximum(np.abs(np.diag(h)), 1e-300)
            edm = abs(0.5 * g @ p)
        if edm < edm_tol:
            converged = True
            break
        lam, accepted = 1.0, False
        for _ in range(max_halvings):
            x1 = np.clip(x + lam * p, lo, hi)
            if combined:
                f1, g1, h1 = yield ("gh", x1)
            else:
                f1, g1 = yield ("grad", x1)
            n_eval += 1
            if np.isfinite(f1) and f1 <= f + f_noise * abs(f):
                accepted = True
                break
            lam *= 0.5
        if not accepted:
            converged = bool(edm < 10.0 * edm_tol)
            break
        x, f, g = x1, f1, g1
        if combined:
            h = h1
    if h is None or (not converged and not combined):
        h = yield ("hess", x)
        n_eval += 1
    try:
        err = np.sqrt(np.abs(np.diag(2.0 * np.linalg.inv(h))))
    except np.linalg.LinAlgError:
        err = np.full(x.size, np.nan)
    return x, err, f, converged, n_eval


class ModelRuntime:
    """The compiled kernels of one model, shared by every fit of it; each fit
    brings only its device columns."""

    def __init__(self, backend: CUDABackend, model: str, kernelT=np.float32):
        self.backend = backend
        self.model = model
        self.spec = load_spec(model)
        self.template = Likelihood(backend, self.spec, kernelT)
        # F + gradient + Hessian in one launch where the model's combined kernel compiles
        self.combined = self.template.combined_kernel()
        self.kernels = {k: b.kernel for k, b in self.template.blocks.items()}
        self.npar = len(self.spec["parameters"])
        self.limits = MODEL_LIMITS[model]
        pre = self.template.pre
        # device bytes per event: raw columns + hoisted columns + prepared copy
        ndim = len(self.spec["dimensions"])
        es = 4 if pre.elem == L.MF_F32 else 8
        hoisted = len(self.spec["event_buffers"]) if self.template.has_precompute else 0
        layout = self.kernels["lh_grad_kernel"].read_layout()
        self.bytes_per_event = ndim * 8 + hoisted * es + layout["bytes_per_event"]
        gk = next(k for k in self.spec["kernels"] if k.get("generate"))
        self.gen = CUDABlock(backend, np.float32 if pre.elem == L.MF_F32 else np.float64)
        self.gen.MakeGenerateKernel(gk["name"], 0, [], gk["outputs"], gk["params"], gk["exprs"], gk["maxprob"],
                                    ranges=list(zip(gk["lo"], gk["hi"])))

    def dataset(self, n: int, seed: int) -> DeviceColumns:
        """Generates the events on the device (up to 65536 xoshiro128++ streams
        seeded independently by SplitMix64, in the storage type of the model's
        precompute input) and returns the columns the likelihood kernels read
        (hoisted by the precompute where the model has one)."""
        pre = self.template.pre
        nseeds = int(min(65536, n))
        self.gen.SetNevents(n)
        # streams seeded on the device (no seed table built or copied);
        # enqueued without a host wait (a thread that gives up is reported by
        # the next synchronous call); the precompute follows in stream order
        self.gen.SubmitGenerateSplitmixAsync(seed, nseeds, -(-n // nseeds))
        raw = self.gen.output
        self.gen.output = DeviceColumns(self.backend, self.gen.elem)
        if not self.template.has_precompute:
            if raw.elem == pre.elem:
                return raw
            cols = DeviceColumns(self.backend, pre.elem)
            cols.upload(raw.download())
            return cols
        if raw.elem != pre.elem:
            src = DeviceColumns(self.backend, pre.elem)
            src.upload(raw.download())
            raw = src
        k = pre.kernel
        out = DeviceColumns(self.backend, pre.elem)
        out.ensure(k.nout, n)
        p = np.zeros(1)
        L.check(L.lib.mf_kernel_store_async(k.handle, raw.buf, raw.stride, n, L.dptr(p), k.nparams, out.buf,
                                            out.stride))
        out._keep = raw  # the generated events stay until the fit's columns go (mf_buffer_free waits for the stream)
        return out

    def param_rows(self, kernel: str, thetas) -> np.ndarray:
        return self.template.param_rows(kernel, np.array(thetas))

    def evaluate(self, kernel: str, datasets, ns, thetas) -> np.ndarray:
        """One batched call: evaluation i reads datasets[i] (ns[i] events) at thetas[i]."""
        k = self.kernels[kernel]
        count = len(datasets)
        rows = np.ascontiguousarray(self.param_rows(kernel, thetas))
        ins = (L.c_buf * count)(*[d.buf for d in datasets])
        strides = np.array([d.stride for d in datasets], dtype=np.uint64)
        nsa = np.array(ns, dtype=np.uint64)
        need = count * k.nout * 8
        if getattr(self, "_out_bytes", 0) < need:  # results buffer, grown as needed and kept
            if getattr(self, "_out", None) is not None:
                L.lib.mf_buffer_free(self._out)
            self._out = L.c_buf()
            self._out_bytes = max(need, 1 << 16)
            L.check(L.lib.mf_buffer_alloc(self.backend.handle, self._out_bytes, C.byref(self._out)))
        u64p = C.POINTER(C.c_uint64)
        # every pending evaluation of the tick in one launch (segments of 2048 events)
        L.check(L.lib.mf_kernel_reduce_multi(k.handle, count, ins, strides.ctypes.data_as(u64p),
                                             nsa.ctypes.data_as(u64p), L.dptr(rows), rows.shape[1], self._out))
        res = np.zeros((count, k.nout))
        L.check(L.lib.mf_buffer_d2h(self._out, 0, res.ctypes.data, res.nbytes))
        return res


@dataclass
class _Active:
    req: FitRequest
    data: DeviceColumns
    bytes: int
    co: object
    pending: tuple
    admitted: float
    result: tuple | None = None


@dataclass
class ServerStats:
    ticks: int = 0
    batched_calls: int = 0
    evaluations: int = 0
    max_active: int = 0
    peak_bytes: int = 0
    outcomes: list = field(default_factory=list)


class FitServer:
    """Continuous batching of fits on one device (see the module docstring).

    ``hbm_budget``: device bytes the resident datasets may take together;
    ``max_active``: slots (fits in flight)."""

    def __init__(self, backend: CUDABackend, hbm_budget: int = 150 << 30, max_active: int = 256,
                 kernelT=np.float32, models=("mass", "spwave")):
        self.backend = backend
        self.budget = hbm_budget
        self.max_active = max_active
        self.models = {m: ModelRuntime(backend, m, kernelT) for m in models}
        # relative precision of -2 ln L: FP32 per-event logs (~6e-8 each) accumulate over the events
        self.f_noise = 2e-7 if np.dtype(kernelT) == np.float32 else 1e-13

    def _hess(self, rt: ModelRuntime, s: np.ndarray) -> np.ndarray:
        """-2 x the Hessian kernel's sums (lower triangle, row by row) as the
        full symmetric matrix: one gather through a flat index map."""
        from .toystudy import _unpack_hessian
        return _unpack_hessian(np.asarray(s)[None, : rt.npar * (rt.npar + 1) // 2], rt.npar)[0]

    def run(self, requests, realtime: bool = True) -> ServerStats:
        """Serves ``requests`` (arrival times relative to the start); with
        ``realtime`` a request is admitted no earlier than its arrival."""
        stats = ServerStats()
        queue = sorted(requests, key=lambda r: r.arrival)
        waiting: list = []  # arrived, not admitted (FIFO)
        active: list[_Active] = []
        used = 0
        t0 = time.perf_counter()
        qi = 0
        while qi < len(queue) or waiting or active:
            now = time.perf_counter() - t0
            while qi < len(queue) and (not realtime or queue[qi].arrival <= now):
                waiting.append(queue[qi])
                qi += 1
            # admission: FIFO while budget and slots allow
            while waiting and len(active) < self.max_active:
                r = waiting[0]
                rt = self.models[r.model]
                need = rt.bytes_per_event * r.nevents
                if used + need > self.budget and active:
                    break
                waiting.pop(0)
                data = rt.dataset(r.nevents, r.seed)
                start = r.start if r.start is not None else np.array(rt.spec["truth"], dtype=np.float64)
                co = newton_fit(start, rt.limits, f_noise=self.f_noise, combined=rt.combined is not None)
                a = _Active(r, data, need, co, co.send(None), time.perf_counter() - t0)
                active.append(a)
                used += need
                stats.peak_bytes = max(stats.peak_bytes, used)
            stats.max_active = max(stats.max_active, len(active))
            if not active:
                if qi < len(queue) and realtime:
                    time.sleep(max(0.0, queue[qi].arrival - (time.perf_counter() - t0)))
                continue
            # one batched call per (model, kernel) over every active fit's pending request
            groups: dict = {}
            for a in active:
                kind, theta = a.pending
                kern = {"hess": "lh_hessian_kernel", "grad": "lh_grad_kernel"}.get(kind) or \
                    self.models[a.req.model].combined
                groups.setdefault((a.req.model, kern), []).append((a, theta))
            for (model, kern), items in groups.items():
                rt = self.models[model]
                sums = rt.evaluate(kern, [a.data for a, _ in items], [a.req.nevents for a, _ in items],
                                   [th for _, th in items])
                stats.batched_calls += 1
                stats.evaluations += len(items)
                npar = rt.npar
                for (a, _), s in zip(items, sums):
                    if kern == "lh_hessian_kernel":
                        reply = self._hess(rt, s)
                    elif kern == "lh_grad_kernel":
                        reply = (-2.0 * s[0], -2.0 * s[1:])
                    else:  # combined: F, gradient, then the Hessian's lower triangle
                        reply = (-2.0 * s[0], -2.0 * s[1:1 + npar], self._hess(rt, s[1 + npar:]))
                    try:
                        a.pending = a.co.send(reply)
                    except StopIteration as stop:
                        a.result = stop.value
            stats.ticks += 1
            done = [a for a in active if a.result is not None]
            now = time.perf_counter() - t0
            for a in done:
                x, err, f, conv, nev = a.result
                arrived = a.req.arrival if realtime else 0.0  # without real time every request is there at 0
                stats.outcomes.append(FitOutcome(a.req.id, a.req.model, a.req.nevents, x, err, f, nev, conv,
                                                 a.admitted, now, now - arrived))
                used -= a.bytes
                a.data.free()
            active = [a for a in active if a.result is None]
        return stats


def poisson_stream(nreq: int, rate_hz: float, seed: int = 1, mass_fraction: float = 0.6, nmin: int = 1000,
                   nmax: int = 5_000_000):
    """Fit requests with Poisson arrivals: 60% mass fits, 40% S+P-wave fits,
    event counts log-uniform in [nmin, nmax]."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate_hz, nreq))
    out = []
    for i in range(nreq):
        model = "mass" if rng.uniform() < mass_fraction else "spwave"
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        out.append(FitRequest(i, model, n, seed * 100003 + i, float(t[i])))
    return out


def latency_summary(stats: ServerStats) -> dict:
    lat = np.array([o.latency for o in stats.outcomes])
    fin = max(o.finished for o in stats.outcomes)
    return {"fits": len(lat), "fits_per_s": len(lat) / fin, "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "max_active": stats.max_active,
            "batched_calls": stats.batched_calls, "evaluations": stats.evaluations,
            "peak_resident_GB": stats.peak_bytes / 1e9,
            "all_converged": bool(all(o.converged for o in stats.outcomes))}
