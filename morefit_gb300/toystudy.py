"""Batched toy studies and batched fits on the device.

The reference runs a toy study as a loop (include/toystudy.hh:55-82): for
every toy it resets the parameters to their start values, draws the event
count (Poisson when the PDF is extended), generates the events with its
generator and fits them with its fitter (Minuit2 MIGRAD + HESSE), then
records the pulls (value - start) / error.

Here all toys are handled at once. The events of every toy come from one
seeded accept-reject generation at the common truth (every toy of the
reference is generated at the same start values as well) and are laid out
back to back, toy s owning events [begin[s], begin[s] + count[s]). One
precompute launch hoists the event-only columns of all toys. The fit is a
batched Newton iteration on F = -2 sum log p: each iteration evaluates F and
its gradient for every active toy in one ragged-segment launch (one block per
toy, mf_kernel_reduce_segments), the Hessian in a second, solves the 8x8
systems on the host (Cholesky vectorised over the toys), and tries the step with a third (F only), halving it per
toy until F does not increase. Parameters are kept inside their limits.
Converged toys (Newton decrement g^T H^-1 g / 2 below ``tol``) leave the
active set. Errors are sqrt(diag(2 H^-1)) at the minimum (errordef 1 on
-2 ln L, as the reference's Minuit2 fit uses).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

import ctypes as C
import math
import re

from . import _lib as L
from .backend import CUDABackend, CUDABlock, DeviceColumns, eval_expressions_batch
from .workloads import DEFAULT_SEED, Likelihood, generate_events, splitmix_seed_rows

# Parameter limits of the K*mumu P-wave fit (Fl in [0, 1], the rest in [-1, 1]),
# as the reference's benchmark drivers declare them.
PWAVE_LIMITS = [(0.0, 1.0)] + [(-1.0, 1.0)] * 7


@dataclass
class FitResult:
    values: np.ndarray      # (ntoys, npar)
    errors: np.ndarray      # (ntoys, npar)
    fmin: np.ndarray        # (ntoys,) -2 ln L at the minimum
    edm: np.ndarray         # (ntoys,) g^T H^-1 g / 2 at the last Newton step
    iterations: np.ndarray  # (ntoys,)
    converged: np.ndarray   # (ntoys,) bool
    evaluations: int        # segment launches issued


class SegmentLikelihood:
    """-2 ln L, gradient and Hessian of many event segments of one device
    event block (toy s: events [begin[s], begin[s] + count[s]))."""

    def __init__(self, like: Likelihood, begins, counts, events_per_block: int = 0):
        """``events_per_block``: 0 evaluates each segment in one block
        (mf_kernel_reduce_segments); n > 0 cuts every segment into runs of n
        events, one block each, combined in a fixed order
        (mf_kernel_reduce_segments_chunked). Either way a segment's sums
        depend on nothing but its own events and parameters."""
        self.like = like
        self.begins = np.ascontiguousarray(begins, dtype=np.uint64)
        self.counts = np.ascontiguousarray(counts, dtype=np.uint32)
        self.params = like.params
        self.events_per_block = int(events_per_block)
        self.evaluations = 0

    def _rows(self, kernel: str, theta: np.ndarray) -> np.ndarray:
        return self.like.param_rows(kernel, theta)

    def _submit(self, kernel: str, idx: np.ndarray, theta: np.ndarray) -> np.ndarray:
        self.evaluations += 1
        parts = self.like.kernel_parts(kernel)
        rows = self._rows(kernel, theta)
        return np.concatenate([self.like.blocks[p].SubmitSegments(self.begins[idx], self.counts[idx], rows,
                                                                  self.events_per_block)
                               for p in parts], axis=1)

    def value(self, idx, theta):
        return -2.0 * self._submit("lh_kernel", idx, theta)[:, 0]

    def value_and_gradient(self, idx, theta):
        s = self._submit("lh_grad_kernel", idx, theta)
        return -2.0 * s[:, 0], -2.0 * s[:, 1:]

    def hessian(self, idx, theta):
        return _unpack_hessian(self._submit("lh_hessian_kernel", idx, theta), theta.shape[1])

    def value_gradient_hessian(self, idx, theta):
        """F, gradient and Hessian per segment: one launch of the combined
        kernel where the model has one, else two."""
        name = self.like.combined_kernel()
        if name is None:
            f, g = self.value_and_gradient(idx, theta)
            return f, g, self.hessian(idx, theta)
        s = self._submit(name, idx, theta)
        npar = theta.shape[1]
        return -2.0 * s[:, 0], -2.0 * s[:, 1:1 + npar], _unpack_hessian(s[:, 1 + npar:], npar)


_TRIL_FULL = {}  # npar -> for each of the npar * npar positions, its index in the packed lower triangle


def _unpack_hessian(s: np.ndarray, npar: int) -> np.ndarray:
    """-2 x the Hessian kernel's sums (row-major lower triangle per row) as
    full symmetric matrices (n, npar, npar): one gather through a flat index
    map (two advanced-index assignments cost several times more)."""
    flat = _TRIL_FULL.get(npar)
    if flat is None:
        i, j = np.tril_indices(npar)
        m = np.empty((npar, npar), dtype=np.intp)
        m[i, j] = np.arange(len(i))
        m[j, i] = np.arange(len(i))
        flat = _TRIL_FULL[npar] = m.ravel()
    return (-2.0 * np.asarray(s))[:, flat].reshape(len(s), npar, npar)


def _spd_solve(h: np.ndarray, g: np.ndarray | None, want_diag: bool = True):
    """Cholesky solves of a batch of symmetric matrices h (n, p, p) in the
    library (mf_spd_solve_batch): (x = h^-1 g or None, diag(h^-1) or None
    when not wanted, ok)."""
    h = np.ascontiguousarray(h, dtype=np.float64)
    n, p, _ = h.shape
    ok = np.zeros(n, dtype=np.uint8)
    dinv = np.zeros((n, p)) if want_diag else None
    x = None
    gp = xp = None
    if g is not None:
        g = np.ascontiguousarray(g, dtype=np.float64)
        x = np.zeros((n, p))
        gp, xp = L.dptr(g), L.dptr(x)
    dp = L.dptr(dinv) if want_diag else None
    L.check(L.lib.mf_spd_solve_batch(n, p, L.dptr(h), gp, xp, dp, ok.ctypes.data_as(C.POINTER(C.c_uint8))))
    return x, dinv, ok.astype(bool)


def _newton_steps(h: np.ndarray, g: np.ndarray) -> np.ndarray:
    """-H^-1 g per toy: Cholesky where H is positive definite, LAPACK's
    pivoted solve for the others."""
    x, _, ok = _spd_solve(h, g, want_diag=False)  # the inverse's diagonal is not needed here
    step = -x
    bad = np.nonzero(~ok)[0]
    if bad.size:
        try:
            step[bad] = -np.linalg.solve(h[bad], g[bad][..., None])[..., 0]
        except np.linalg.LinAlgError:
            for t in bad:
                step[t] = -np.linalg.lstsq(h[t], g[t], rcond=None)[0]
    return step


def _inverse_diagonal(h: np.ndarray) -> np.ndarray:
    """diag(H^-1) per toy: from the Cholesky factor where H is positive
    definite, LAPACK's inverse for the others."""
    _, diag, ok = _spd_solve(h, None)
    bad = np.nonzero(~ok)[0]
    if bad.size:
        diag[bad] = np.einsum("tii->ti", np.linalg.inv(h[bad]))
    return diag


def fit_segments(sl: SegmentLikelihood, theta0: np.ndarray, limits, tol: float = 1e-9, max_iter: int = 50,
                 max_halvings: int = 30) -> FitResult:
    """Batched damped Newton minimisation of every segment's -2 ln L."""
    theta = np.array(theta0, dtype=np.float64, copy=True)
    ntoy, npar = theta.shape
    lo = np.array([l for l, _ in limits])
    hi = np.array([h for _, h in limits])
    iters = np.zeros(ntoy, dtype=np.int64)
    edm = np.full(ntoy, np.inf)
    conv = np.zeros(ntoy, dtype=bool)
    fmin = np.full(ntoy, np.nan)
    active = np.arange(ntoy)
    for _ in range(max_iter):
        if active.size == 0:
            break
        th = theta[active]
        f, g, h = sl.value_gradient_hessian(active, th)
        fmin[active] = f
        step = _newton_steps(h, g)
        dec = -0.5 * np.einsum("ij,ij->i", g, step)
        # a Hessian that is not positive definite: fall back to a scaled gradient step
        bad = ~(dec > 0) | ~np.isfinite(dec)
        if bad.any():
            scale = 1.0 / np.maximum(np.abs(np.einsum("tii->ti", h[bad])), 1e-300)
            step[bad] = -g[bad] * scale
            dec[bad] = np.abs(0.5 * np.einsum("ij,ij->i", g[bad], step[bad]))
        edm[active] = dec
        iters[active] += 1
        done = dec < tol
        conv[active[done]] = True
        # step with halving, per toy, for those not yet converged
        todo = np.nonzero(~done)[0]
        lam = np.ones(len(todo))
        pending = np.arange(len(todo))
        for _ in range(max_halvings):
            if pending.size == 0:
                break
            rows = todo[pending]
            trial = np.clip(th[rows] + lam[pending, None] * step[rows], lo, hi)
            ft = sl.value(active[rows], trial)
            ok = np.isfinite(ft) & (ft <= f[rows] + 1e-12 * np.abs(f[rows]))
            theta[active[rows[ok]]] = trial[ok]
            pending = pending[~ok]
            lam[pending] *= 0.5
        active = active[~done]
    # errors from the Hessian at the final point
    idx = np.arange(ntoy)
    f, g, h = sl.value_gradient_hessian(idx, theta)
    fmin[:] = f
    errors = np.sqrt(np.abs(2.0 * _inverse_diagonal(h)))
    return FitResult(theta, errors, fmin, edm, iters, conv, sl.evaluations)


def _log_argument(expr: str):
    """X when ``expr`` is exactly log(X) (one top-level logarithm), else None."""
    if not (expr.startswith("log(") and expr.endswith(")")):
        return None
    depth = 0
    for i, ch in enumerate(expr[3:], start=3):
        depth += ch == "("
        depth -= ch == ")"
        if depth == 0:
            return expr[4:-1] if i == len(expr) - 1 else None
    return None


def density_expression(spec: dict):
    """The model's density as one expression of the raw observables with the
    fitter's parameters: exp of the log-density kernel text (the lh kernel,
    fitter.hh:380-396) with every hoisted event buffer replaced by its own
    expression. A log-density that is one logarithm, log(X), gives X itself:
    the same density where X > 0, and where X <= 0 both forms reject every
    proposal (exp(log X) is NaN or 0 there), without a NaN that would send
    the generator's fast accept test to its exact FP64 path. Returns
    (expression, parameter names, parameter-buffer list)."""
    k = next(k for k in spec["kernels"] if k["name"] == "lh_kernel")
    expr = k["exprs"][0]
    for name, e in sorted(spec["event_buffers"], key=lambda x: -len(x[0])):
        if name != e:
            expr = re.sub(r"\b" + re.escape(name) + r"\b", "(" + e + ")", expr)
    inner = _log_argument(expr)
    return (inner if inner is not None else "exp(" + expr + ")"), list(k["params"]), spec["lh_buffers"]


def pwave_maxprob(theta: np.ndarray) -> np.ndarray:
    """KstarmumuAngularPDF::get_max (physicspdfs.hh:209-213) for each row of theta
    (Fl, S3, S4, S5, Afb, S7, S8, S9)."""
    t = np.abs(np.asarray(theta, dtype=np.float64))
    return 9.0 / 32.0 / math.pi * (4.0 + t[:, 1] + t[:, 2] + t[:, 3] + 4.0 / 3.0 * t[:, 4] + t[:, 5] + t[:, 6]
                                   + t[:, 7])


def generate_segments(backend: CUDABackend, spec: dict, theta: np.ndarray, counts, maxprob: np.ndarray,
                      seed: int = DEFAULT_SEED, threads_per_seg: int = 16) -> DeviceColumns:
    """Events of many datasets, dataset s at parameters theta[s] (one launch):
    dataset s owns events [begin[s], begin[s] + counts[s]) of the returned block.
    Stream r of segment s is seeded independently (SplitMix64 of seed and the
    stream's index), so a segment's events depend only on its own streams."""
    expr, params, bufs = density_expression(spec)
    gk = next(k for k in spec["kernels"] if k.get("generate"))
    cache = backend.__dict__.setdefault("_gen_segment_blocks", {})  # built once per backend and model
    blk = cache.get((spec["workload"], expr))
    if blk is None:
        blk = CUDABlock(backend, np.float64)
        blk.MakeGenerateKernel("gen_segments", 0, [], gk["outputs"], params, [expr], 1.0,
                               ranges=list(zip(gk["lo"], gk["hi"])))
        cache[(spec["workload"], expr)] = blk
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    nfloat = theta.shape[1]
    rows = theta if len(params) == nfloat else np.concatenate(
        [theta, eval_expressions_batch(params[:nfloat], theta, [e for _, e in bufs])], axis=1)
    counts = np.ascontiguousarray(counts, dtype=np.uint32)
    begins = np.concatenate([[0], np.cumsum(counts, dtype=np.uint64)[:-1]]).astype(np.uint64)
    nseg = len(counts)
    nthreads = nseg * threads_per_seg
    seeds = np.ascontiguousarray(splitmix_seed_rows(nthreads, seed), dtype=np.uint32)
    out = DeviceColumns(backend, L.MF_F64)
    out.ensure(len(gk["outputs"]), int(counts.sum()))
    mp = np.ascontiguousarray(maxprob, dtype=np.float64)
    per = int(-(-int(counts.max()) // threads_per_seg))
    L.check(L.lib.mf_kernel_generate_segments(
        blk.kernel.handle, seeds.ctypes.data_as(C.POINTER(C.c_uint32)), nthreads, threads_per_seg, nseg,
        begins.ctypes.data_as(C.POINTER(C.c_uint64)), counts.ctypes.data_as(C.POINTER(C.c_uint32)),
        L.dptr(np.ascontiguousarray(rows)), rows.shape[1], L.dptr(mp), out.buf, out.stride, 10000 * per))
    return out


@dataclass
class ToyResult:
    counts: np.ndarray
    fit: FitResult
    truth: np.ndarray       # (ntoys, npar)
    pulls: np.ndarray       # (ntoys, npar)
    timing: dict


@dataclass(frozen=True)
class SegmentSchedule:
    """How the ragged-segment kernels cover the toys: ``block`` threads per
    block; ``events_per_block`` 0 = one block per segment (each thread
    strides over its segment), else runs of that many events per block
    (``events_per_block / block`` events per thread) combined per segment."""
    block: int
    events_per_block: int = 0

    def __str__(self) -> str:
        return f"b{self.block}" + (f"_e{self.events_per_block}" if self.events_per_block else "_seg")


DEFAULT_SCHEDULE = SegmentSchedule(256, 0)

# Tuned schedules of this process: (model, kernel type, device, log2 of the
# median and of the largest segment size, log2 of the toy count) -> schedule.
# With MOREFIT_GB300_CACHE set they are also kept in
# $MOREFIT_GB300_CACHE/toy_schedules.json and read back by later processes.
_SCHEDULES: dict = {}


def _schedule_file():
    import os
    d = os.environ.get("MOREFIT_GB300_CACHE")
    return None if not d else os.path.join(d, "toy_schedules.json")


def _load_schedules() -> dict:
    import json
    f = _schedule_file()
    if f is None:
        return {}
    try:
        with open(f) as fh:
            return {k: SegmentSchedule(int(v[0]), int(v[1])) for k, v in json.load(fh).items()}
    except (OSError, ValueError, TypeError, IndexError):
        return {}


def _store_schedule(key: str, sched: SegmentSchedule) -> None:
    import json
    import os
    f = _schedule_file()
    if f is None:
        return
    table = {k: [v.block, v.events_per_block] for k, v in _load_schedules().items()}
    table[key] = [sched.block, sched.events_per_block]
    os.makedirs(os.path.dirname(f), exist_ok=True)
    tmp = f"{f}.{os.getpid()}"
    with open(tmp, "w") as fh:
        json.dump(table, fh, indent=1, sort_keys=True)
    os.replace(tmp, f)


def size_histogram_key(counts) -> tuple:
    """The segment-size histogram a schedule is tuned for, coarsened to
    powers of two: (median size, largest size, number of segments)."""
    c = np.asarray(counts)
    b = lambda x: int(round(math.log2(max(float(x), 1.0))))
    return (b(np.median(c)), b(c.max()), b(len(c)))


class ToyStudy:
    """Toy studies of one model (reference include/toystudy.hh:40-115).

    ``toy(nruns, nevents)`` generates ``nruns`` datasets at the truth values
    and fits each, starting from the truth. With ``poisson=True`` the event
    counts are Poisson(nevents) from a seeded generator, clipped to
    ``clip``; otherwise every toy has ``nevents`` events (the reference draws
    Poisson counts only for extended PDFs)."""

    # threads per block tried for the segment kernels
    BLOCK_CANDIDATES = (64, 128, 256)
    # events per thread tried for the chunked entry (runs of block x this many
    # events); runs as long as the largest segment are left out
    EVENTS_PER_THREAD_CANDIDATES = (2, 4, 8, 16)
    TUNE_MIN_TOYS = 512

    def __init__(self, backend: CUDABackend, spec: dict, kernelT=np.float64, limits=None,
                 seed: int = DEFAULT_SEED, generator_threads: int = 65536, block: int = 0,
                 schedule: SegmentSchedule | None = None):
        """``schedule`` (or ``block``: threads per segment, one block per
        segment) fixes how the segment kernels run. Otherwise a study of at
        least TUNE_MIN_TOYS toys takes the schedule tuned for its model,
        kernel type, device and segment-size histogram: from this process's
        table (or the MOREFIT_GB300_CACHE file), else measured there and
        then (the candidate whose Newton-iteration launches, F + gradient +
        Hessian and one F trial over that study's toys, take the least
        time) and stored. Smaller studies without a stored schedule run
        DEFAULT_SCHEDULE."""
        self.backend = backend
        self.spec = spec
        self.kernelT = kernelT
        self.limits = limits if limits is not None else PWAVE_LIMITS
        self.seed = seed
        self.generator_threads = generator_threads
        if schedule is None and block:
            schedule = SegmentSchedule(block, 0)
        self.fixed = schedule
        self.schedule = schedule or DEFAULT_SCHEDULE
        self.tuning = None
        self._likes = {}

    @property
    def block(self) -> int:
        return self.schedule.block

    def _likelihood(self, block: int) -> Likelihood:
        if block not in self._likes:  # kernels built once per block size
            self._likes[block] = Likelihood(self.backend, self.spec, self.kernelT, block=block)
        return self._likes[block]

    def _schedule_key(self, counts) -> str:
        dev = self.backend.__dict__.get("_device_key")
        if dev is None:
            p = self.backend.properties()
            dev = self.backend._device_key = f"{p['name']}:{p['sms']}"
        return "|".join([str(self.spec.get("workload", "model")), np.dtype(self.kernelT).name, dev,
                         ",".join(map(str, size_histogram_key(counts)))])

    def candidates(self, counts) -> list:
        """Schedules the tuner measures for segments of these sizes."""
        cmax = int(np.max(counts))
        out = []
        for blk in self.BLOCK_CANDIDATES:
            out.append(SegmentSchedule(blk, 0))
            for e in self.EVENTS_PER_THREAD_CANDIDATES:
                if blk * e < cmax:
                    out.append(SegmentSchedule(blk, blk * e))
        return out

    def _choose(self, cols, begins, counts, truth) -> None:
        if self.fixed is not None:
            return
        key = self._schedule_key(counts)
        if key not in _SCHEDULES:
            _SCHEDULES.update({k: v for k, v in _load_schedules().items() if k not in _SCHEDULES})
        if key in _SCHEDULES:
            self.schedule = _SCHEDULES[key]
            self.tuning = {"schedule": str(self.schedule), "cached": True, "key": key}
        elif len(counts) >= self.TUNE_MIN_TOYS:
            self._tune(cols, begins, counts, truth, key)
        else:
            self.schedule = DEFAULT_SCHEDULE

    def _tune(self, cols, begins, counts, truth, key) -> None:
        import time
        idx = np.arange(len(counts))
        times = {}
        for sched in self.candidates(counts):
            like = self._likelihood(sched.block)
            like.set_device_data(cols)
            sl = SegmentLikelihood(like, begins, counts, sched.events_per_block)
            # once to build the kernels and the prepared copy, then timed
            sl.value_gradient_hessian(idx, truth)
            sl.value(idx, truth)
            best = math.inf
            for _ in range(3):
                t0 = time.perf_counter()
                sl.value_gradient_hessian(idx, truth)
                sl.value(idx, truth)
                best = min(best, time.perf_counter() - t0)
            times[sched] = best
        self.schedule = min(times, key=times.get)
        _SCHEDULES[key] = self.schedule
        _store_schedule(key, self.schedule)
        self.tuning = {"schedule": str(self.schedule), "cached": False, "key": key, "toys": len(counts),
                       "launch_s": {str(k): v for k, v in times.items()}}

    def serial_fits_per_s(self, result: "ToyResult", ntoys: int = 32) -> float:
        """The per-fit serial baseline: the first ``ntoys`` toys of ``result``'s
        event block fitted one at a time (one segment per launch, each fit
        waiting for the previous), same fitter and tolerances."""
        import time
        sl_all = self._last_segments
        t0 = time.perf_counter()
        for t in range(min(ntoys, len(result.counts))):
            sl = SegmentLikelihood(sl_all.like, sl_all.begins[t:t + 1], sl_all.counts[t:t + 1], sl_all.events_per_block)
            fit_segments(sl, result.truth[t:t + 1], self.limits)
        return min(ntoys, len(result.counts)) / (time.perf_counter() - t0)

    def toy(self, nruns: int, nevents: int, poisson: bool = False, clip=(1, None), jitter: float = 0.0,
            maxprob=pwave_maxprob) -> ToyResult:
        """``jitter``: each toy's truth is the model truth times (1 + u), u
        uniform in [-jitter, jitter] (zero truths stay zero); such toys are
        generated one dataset per segment, each at its own truth, with the
        bound ``maxprob(theta)`` per toy (the P-wave's get_max by default)."""
        import time
        t0 = time.perf_counter()
        rng = np.random.default_rng(self.seed)
        if poisson:
            counts = rng.poisson(nevents, nruns)
        else:
            counts = np.full(nruns, nevents)
        counts = np.clip(counts, clip[0], clip[1] if clip[1] is not None else np.iinfo(np.int64).max)
        begins = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint64)
        total = int(counts.sum())
        base = np.array(self.spec["truth"], dtype=np.float64)
        if jitter > 0.0:
            truth = base * (1.0 + rng.uniform(-jitter, jitter, (nruns, base.size)))
            cols = generate_segments(self.backend, self.spec, truth, counts, maxprob(truth), seed=self.seed)
        else:
            truth = np.tile(base, (nruns, 1))
            cols = generate_events(self.backend, self.spec, total, seed=self.seed,
                                   max_workitems=self.generator_threads, kernelT=np.float64)
        self._choose(cols, begins, counts, truth)
        like = self._likelihood(self.schedule.block)
        like.set_device_data(cols)
        self.backend.synchronize()
        t1 = time.perf_counter()
        sl = SegmentLikelihood(like, begins, counts, self.schedule.events_per_block)
        self._last_segments = sl
        fit = fit_segments(sl, truth, self.limits)
        t2 = time.perf_counter()
        pulls = (fit.values - truth) / fit.errors
        return ToyResult(counts, fit, truth, pulls,
                         {"generate_precompute_s": t1 - t0, "fit_s": t2 - t1, "total_s": t2 - t0})
