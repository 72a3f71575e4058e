#!/usr/bin/env python3
"""Benchmark: K*mumu P-wave NLL + analytic gradient evaluations per second at 1M events.

One step = one evaluation of sum log p and its 8 gradient sums over the 1M
events of one dataset: the lh_grad kernel of the reference's fitter
(include/fitter.hh:1054-1151) lowered to CUDA on sm_103a.

  value  : device throughput, FP64, the hoisted event columns resident in HBM,
           timed with CUDA events on the backend's stream. Datasets rotate
           over enough independent 1M-event sets that the bytes read between
           two reads of one set exceed twice the L2 (129 MB).
  e2e    : the same metric through the public API with HOST event buffers:
           every step uploads the raw events (3 x 1M FP64 from pinned host
           memory), runs the precompute kernel and the NLL+gradient kernel,
           and reads the 9 sums back.
  mixed  : FP32 storage/per-event arithmetic with FP64 sums (same timing as value).
  cpu_baseline : the reference's kernel text (the same get_kernel() strings)
           compiled with gcc, on the host cores, Kahan-summed as the
           reference's CPU backend does (oracle/spec_kernel.py).

--impl reference times only that CPU path (all host threads).
"""
from __future__ import annotations

import argparse
import datetime
import json
import math
import os
import platform
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "K*mumu P-wave NLL+grad evals/s at 1M events"
N_EVENTS = 1_000_000
L2_BYTES = 129 * 1024 * 1024


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


# dram__bytes_read.sum + dram__bytes_write.sum of one lh_grad launch (FP64
# storage, double-float arithmetic, 9 prepared columns, 1M events) from the
# full ncu capture summarised in profiles/mf_reduce_part_lh_grad_pwave_1M.md
# (mf_reduce_part: the entry batched evaluations launch).
NCU_TRAFFIC_F64 = 72.349440e6 + 0.755968e6
NCU_TRAFFIC_SOURCE = "ncu --set full, one mf_reduce_part launch, profiles/mf_reduce_part_lh_grad_pwave_1M.md"
# evaluations per combine launch of mf_kernel_reduce_many (mf_runtime.cpp, launch_batched)
COMBINE_CHUNK = 256
# contexts the end-to-end steps rotate over
E2E_LANES = 4


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 50 ms by one
    background nvidia-smi process; summary() keeps the samples stamped inside
    the timed region (mark_start/mark_end)."""

    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self._proc = None
        self._file = None
        self.t0 = self.t1 = None

    def __enter__(self):
        import tempfile
        self._file = tempfile.TemporaryFile(mode="w+")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                           "--format=csv,noheader,nounits", "-lms", "50"],
                                          stdout=self._file, stderr=subprocess.DEVNULL)
            time.sleep(0.5)  # first sample before the timed region starts
        except Exception:
            self._proc = None
        return self

    def mark_start(self):
        self.t0 = datetime.datetime.now()

    def mark_end(self):
        self.t1 = datetime.datetime.now()

    def __exit__(self, *a):
        if self._proc is not None:
            time.sleep(0.1)
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()

    def summary(self):
        rows = []
        if self._file is not None:
            self._file.seek(0)
            for line in self._file:
                f = [x.strip() for x in line.split(",")]
                if len(f) < 8:
                    continue
                try:
                    ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f")
                except ValueError:
                    continue
                rows.append((ts, f[1:]))
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        inside = [r for ts, r in rows if self.t0 and self.t1 and self.t0 <= ts <= self.t1]
        window = "timed region"
        if not inside:  # region shorter than the sampling period: nearest samples
            inside = [r for _, r in rows]
            window = "whole run (timed region shorter than a sample)"
        num = lambda v: v.replace(".", "", 1).isdigit()
        sm = [float(s[0]) for s in inside if num(s[0])]
        mx = [float(s[1]) for s in inside if num(s[1])]
        pw = [float(s[2]) for s in inside if num(s[2])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in inside for i in range(4) if s[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w": statistics.median(pw) if pw else None, "reasons": reasons,
                "samples": len(inside), "window": window}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_value(ms: float, steps: int):
    """Whole-job rate of N independent replicas: the slowest rank's time
    (all-reduce MAX over the process group, when there is one) and
    world x steps evaluations per second of it. Returns (ms, value)."""
    import torch
    import torch.distributed as dist
    world = 1
    if dist.is_available() and dist.is_initialized():
        world = dist.get_world_size()
        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([ms], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * steps / (ms / 1e3)


def bench_config(n: int) -> dict:
    """The workload both arms name (identical dicts): the K*mumu P-wave events
    of dataset 0 (seed 229387429, the reference's accelerator partition of
    8192 generator streams) and the GPU arm's L2 policy."""
    nsets = rotation_sets(n)
    return {"workload": "K*mumu P-wave angular fit, 8 free parameters, 1M events, FP64",
            "nevents": n, "events": "seeded accept-reject, seed 229387429, accelerator partition (8192 streams)",
            "l2": f"GPU arm: {nsets} datasets x {n * 72 / 1e6:.0f} MB read in rotation (> 2x L2), no flush",
            "parallelism": "single device"}


def rotation_sets(n: int) -> int:
    """Independent 1M-event datasets the device arm rotates over so that the
    bytes read between two reads of one set exceed twice the L2."""
    return max(2, math.ceil(2 * L2_BYTES / (n * 11 * 8)) + 1)


def _refkit():
    p = ROOT / "oracle" / "_ref" / platform.machine() / "refkit"
    return p if p.exists() else None


def cpu_reference_rate(events: np.ndarray, nthreads: int, max_evals: int, seconds: float) -> dict:
    """NLL + gradient evaluations per second of the reference's CPU path over
    `events` (3 x n P-wave events) at the truth, on `nthreads` host threads:
    the reference's own fitter::likelihood_and_gradient over its CPU backend's
    loop (oracle/_ref/<arch>/refkit benchevents: the reference compiled from
    its sources, its kernel text compiled by gcc), "kind": "reference"; where
    the kit is not built, the reference's lh_grad kernel text in the oracle's
    restatement of that loop (oracle/spec_kernel.py), "kind": "port".
    At most max_evals evaluations or `seconds` of them, after 3 untimed ones."""
    import tempfile
    kit = _refkit()
    if kit is not None:
        with tempfile.TemporaryDirectory() as td:
            path = Path(td) / "events.f64"
            np.ascontiguousarray(events, dtype=np.float64).tofile(path)
            r = subprocess.run([str(kit), "benchevents", "pwave", str(path), str(nthreads), str(max_evals),
                                str(seconds)], capture_output=True, text=True, check=True)
        d = json.loads(r.stdout.strip().splitlines()[-1])
        return {"value": d["evals_per_s"], "nthreads": nthreads, "nevals": d["nevals"], "seconds": d["seconds"],
                "nll": d["nll"], "kind": "reference",
                "how": "the reference's fitter::likelihood_and_gradient over its CPU backend loop (kernel text "
                       "compiled by gcc -O3), oracle/_ref refkit benchevents"}
    from oracle.spec_kernel import SpecKernel
    g = json.loads((ROOT / "tests" / "golden" / "pwave_n1000000.json").read_text())
    ks = {k["name"]: k for k in g["kernels"]}
    cols = SpecKernel(ks["precompute_kernel"]).store(events, [])
    grad = SpecKernel(ks["lh_grad_kernel"])
    pv = np.array(g["points"][0]["kernel_params"]["lh_grad_kernel"])  # the truth
    for _ in range(3):
        grad.reduce(cols, pv, nthreads)
    t0 = time.perf_counter()
    done = 0
    while done < max_evals and (done == 0 or time.perf_counter() - t0 < seconds):
        s = grad.reduce(cols, pv, nthreads)
        done += 1
    dt = time.perf_counter() - t0
    return {"value": done / dt, "nthreads": nthreads, "nevals": done, "seconds": dt, "nll": float(-2.0 * s[0]),
            "kind": "port", "how": "the reference's lh_grad kernel text compiled by gcc -O3 in the oracle's "
                                   "restatement of its CPU backend loop (oracle/spec_kernel.py)"}


def reference_arm(args):
    """The reference's CPU path on the events of the device arm's dataset 0,
    all host threads (the line's value) and one thread (every reference
    driver's setting, benchmarking/morefit_kstarmumu.cc:27) beside it."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import mforacle
    n = args.nevents
    nper, nseeds = mforacle.accelerator_partition(n)
    ev = mforacle.generate_partitioned("pwave", n, nper, nseeds)
    h = mforacle.fnv1a(ev)
    cores = os.cpu_count() or 1
    allc = cpu_reference_rate(ev, cores, args.steps, args.cpu_seconds)
    one = cpu_reference_rate(ev, 1, args.steps, args.cpu_seconds)
    v = allc["value"]
    line = {"metric": METRIC, "value": v, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "steps_timed": allc["nevals"], "warmup": args.warmup, "ms_per_step": 1e3 / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded accept-reject K*mumu P-wave events (the device arm's dataset 0)",
            "impl": "reference", "config": bench_config(n),
            "cpu_baseline": {"value": v, "unit": "evals/s", "cores": cores, "kind": allc["kind"],
                             "sample": f"{allc['nevals']} NLL+grad evaluations over all {n} events (at most K or "
                                       f"{args.cpu_seconds:g} s); {allc['how']}"},
            "nthreads_1": {"value": one["value"], "unit": "evals/s", "cores": 1, "nevals": one["nevals"],
                           "nll": one["nll"]},
            "events_fnv1a": h, "nll": allc["nll"],
            "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def ours(args):
    import ctypes as C
    import torch
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import CUDABackend
    from morefit_gb300.workloads import Likelihood, generate_events, load_spec

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    backend = CUDABackend(local)
    spec = load_spec("pwave")
    truth = np.array(spec["truth"])
    n = args.nevents
    ks = {k["name"]: k for k in spec["kernels"]}

    def make_sets(kernelT, native=False):
        """Rotating datasets totalling more than 2x L2 of what the NLL+grad kernel reads
        (dataset r: seed 229387429 + 1000 rank + r). Returns the sets, the kernel's
        algorithmic bytes per launch (columns it reads x n x element bytes) and the
        number of sets."""
        nsets = rotation_sets(n) if kernelT == np.float64 else max(2, math.ceil(2 * L2_BYTES / (n * 11 * 4)) + 1)
        sets = []
        for r in range(nsets):
            like = Likelihood(backend, spec, kernelT, native_f64=native)
            cols = generate_events(backend, spec, n, seed=229387429 + 1000 * rank + r)
            like.set_device_data(cols)
            sets.append(like)
        layout = sets[0].blocks["lh_grad_kernel"].kernel.read_layout()
        return sets, n * layout["bytes_per_event"], nsets

    stream_ptr = C_stream(backend)
    ext = torch.cuda.ExternalStream(stream_ptr, device=torch.device("cuda", local))

    def timed_device(sets, K, W, clk=None):
        """K NLL+grad evaluations rotating over the datasets through one
        mf_kernel_reduce_many call (the batched entry: parameter-only values
        evaluated per evaluation, launches enqueued back to back), bracketed by
        CUDA events on the library's stream. The call's argument arrays (input
        handles, strides, sizes, one parameter row per evaluation) are built
        before the first event; everything the library does is inside."""
        import ctypes as C
        pv = sets[0].param_vector("lh_grad_kernel", truth)
        kern = sets[0].blocks["lh_grad_kernel"].kernel
        out_buf = L.c_buf()
        L.check(L.lib.mf_buffer_alloc(backend.handle, max(K, W, len(sets), 1) * kern.nout * 8, C.byref(out_buf)))
        u64p = C.POINTER(C.c_uint64)

        def request(count):
            """The call's arguments, marshalled for ctypes (the arrays are kept
            alive by the returned tuple)."""
            ins = (L.c_buf * count)(*[sets[i % len(sets)].blocks["lh_grad_kernel"].input.buf for i in range(count)])
            strides = np.array([sets[i % len(sets)].blocks["lh_grad_kernel"].input.stride for i in range(count)],
                               dtype=np.uint64)
            ns = np.full(count, n, dtype=np.uint64)
            rows = np.ascontiguousarray(np.tile(pv, (count, 1)))
            args = (kern.handle, count, ins, strides.ctypes.data_as(u64p), ns.ctypes.data_as(u64p), L.dptr(rows),
                    len(pv), out_buf)
            return args, (strides, ns, rows)

        def enqueue(req):
            L.check(L.lib.mf_kernel_reduce_many(*req[0]))

        # one untimed launch per dataset first: each makes the dataset's
        # prepared columns (folded, pre-split) that the kernel reads
        enqueue(request(len(sets)))
        enqueue(request(W))
        timed = request(K)
        backend.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if clk is not None:
            clk.mark_start()
        e0.record(ext)
        enqueue(timed)
        e1.record(ext)
        e1.synchronize()
        if clk is not None:
            clk.mark_end()
        backend.synchronize()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        res = np.zeros(kern.nout)
        L.check(L.lib.mf_buffer_d2h(out_buf, 0, res.ctypes.data, kern.nout * 8))
        L.lib.mf_buffer_free(out_buf)
        return ms, res

    # ---------------- FP64 device throughput (value) ----------------
    sets64, bytes64, nsets64 = make_sets(np.float64)
    with ClockSampler(local) as clk:
        ms64, res64 = timed_device(sets64, args.steps, args.warmup, clk)
    ms64, value = replica_value(ms64, args.steps)
    avg_launch_s = ms64 / 1e3 / args.steps
    hbm_peak, peak_kind = _peaks()
    achieved = bytes64 / avg_launch_s / 1e9

    # ---------------- native FP64 arithmetic (reported beside the default) ----------------
    native = None
    if not args.no_native:
        setsn, _, _ = make_sets(np.float64, native=True)
        msn, resn = timed_device(setsn, max(50, args.steps // 10), args.warmup)
        native = {"value": world * max(50, args.steps // 10) / (msn / 1e3), "unit": "evals/s",
                  "dtype": "f64 storage, native FP64 arithmetic",
                  "rel_diff_vs_default": float(np.max(np.abs(resn - res64) / np.maximum(np.abs(res64), 1.0)))}
        del setsn

    # ---------------- mixed precision ----------------
    mixed = None
    if not args.no_mixed:
        sets32, bytes32, _ = make_sets(np.float32)
        # K-step timings of either precision alternated five times, medians:
        # at K = 20 one timing is ~0.2 ms and its fixed part (first launch,
        # final combine) varies from run to run
        t64, t32 = [], []
        for _ in range(5):
            t64.append(timed_device(sets64, args.steps, args.warmup)[0])
            m, res32 = timed_device(sets32, args.steps, args.warmup)
            t32.append(m)
        ms32, ms64p = statistics.median(t32), statistics.median(t64)
        mixed = {"value": world * args.steps / (ms32 / 1e3), "unit": "evals/s", "dtype": "f32 storage+arith, f64 sums",
                 "speedup_vs_f64": ms64p / ms32, "timing": "median of 5 K-step timings, alternated with FP64's",
                 "f64_us_per_eval_paired": 1e3 * ms64p / args.steps,
                 "speedup_vs_native_f64": (msn / max(50, args.steps // 10)) / (ms32 / args.steps) if native else None,
                 "roofline": {"bound": "hbm", "achieved": bytes32 / (ms32 / 1e3 / args.steps) / 1e9,
                              "peak": hbm_peak, "unit": "GB/s",
                              "frac": bytes32 / (ms32 / 1e3 / args.steps) / 1e9 / hbm_peak},
                 "nll_rel_diff_vs_f64": abs(res32[0] - res64[0]) / abs(res64[0])}
        del sets32

    # ---------------- e2e through the public API, host buffers ----------------
    # Every step uploads the raw events (3 FP64 columns) from page-locked host
    # memory, runs the precompute, prepares the columns, evaluates NLL+grad and
    # reads the sums back into host memory. Pipelined: steps rotate over
    # E2E_LANES contexts (own stream and scratch each), so one step's upload
    # overlaps earlier steps' kernels; the host waits only before reusing a
    # context's buffers and at the end. The upload (24 MB at the measured
    # 207 GB/s of page-locked host-to-device copies, one stream or several)
    # bounds the step at about 116 us; four lanes come within 2% of it.
    if args.no_e2e:
        args.e2e_steps = 3
    host = sets64[0].pre.input.download()  # (3, n) FP64 raw events of set 0
    pinned = torch.empty(host.shape, dtype=torch.float64).pin_memory()
    pinned.numpy()[...] = host
    host_pinned = pinned.numpy()
    ke = max(3, min(args.steps, args.e2e_steps))
    nout = 1 + len(spec["parameters"])
    res_t = torch.zeros((max(ke, args.warmup, E2E_LANES), nout), dtype=torch.float64).pin_memory()
    res = res_t.numpy()
    lanes = []
    for b in [backend] + [CUDABackend(local) for _ in range(E2E_LANES - 1)]:
        lk = Likelihood(b, spec, np.float64)
        ob = L.c_buf()
        L.check(L.lib.mf_buffer_alloc(b.handle, nout * 8, C.byref(ob)))
        lanes.append((b, lk, ob))

    def e2e_run(k):
        for i in range(k):
            b, lk, ob = lanes[i % E2E_LANES]
            if i >= E2E_LANES:
                b.synchronize()  # this context's previous step is done: its buffers may be reused
            lk.set_data_async(host_pinned)
            lk.sums_async("lh_grad_kernel", truth, ob, 0)
            L.check(L.lib.mf_buffer_d2h_async(ob, 0, res[i].ctypes.data, nout * 8))
        for b, _, _ in lanes:
            b.synchronize()

    e2e_run(args.warmup)
    t0 = time.perf_counter()
    e2e_run(ke)
    e2e_s = (time.perf_counter() - t0) / ke
    e2e_rel = float(np.max(np.abs(res[:ke, 0] - res64[0])) / abs(res64[0]))

    # the same steps with the raw events read in place from page-locked host
    # memory by the precompute kernel (no separate copy to HBM)
    def e2e_mapped_run(k):
        for i in range(k):
            b, lk, ob = lanes[i % E2E_LANES]
            if i >= E2E_LANES:
                b.synchronize()
            lk.set_data_mapped(host_pinned)
            lk.sums_async("lh_grad_kernel", truth, ob, 0)
            L.check(L.lib.mf_buffer_d2h_async(ob, 0, res[i].ctypes.data, nout * 8))
        for b, _, _ in lanes:
            b.synchronize()

    e2e_mapped_run(args.warmup)
    t0 = time.perf_counter()
    e2e_mapped_run(ke)
    e2e_mapped_s = (time.perf_counter() - t0) / ke
    e2e_mapped_rel = float(np.max(np.abs(res[:ke, 0] - res64[0])) / abs(res64[0]))
    # sequential form: one step at a time, each waiting for its result (latency)
    like = lanes[0][1]
    for _ in range(3):
        like.set_data(host_pinned)
        like.likelihood_and_gradient(truth)
    t0 = time.perf_counter()
    for _ in range(ke):
        like.set_data(host_pinned)
        nll_e2e, g_e2e = like.likelihood_and_gradient(truth)
    seq_s = (time.perf_counter() - t0) / ke
    # fit-loop form: events resident, parameters in / sums out per evaluation
    t0 = time.perf_counter()
    for _ in range(ke * 4):
        like.likelihood_and_gradient(truth)
    fit_loop_s = (time.perf_counter() - t0) / (ke * 4)
    for b, lk, ob in lanes:
        L.lib.mf_buffer_free(ob)

    # ---------------- S+P wave with acceptance, 10M events, mixed precision ----------------
    spw = None
    if not args.no_spwave:
        spec3 = load_spec("spwave")
        n3 = args.spwave_events
        truth3 = np.array(spec3["truth"])
        cols3 = generate_events(backend, spec3, n3, seed=229387429 + 1000 * rank)
        l32 = Likelihood(backend, spec3, np.float32)
        l32.set_device_data(cols3)
        l64 = Likelihood(backend, spec3, np.float64)
        l64.set_device_data(cols3)
        del cols3

        def timed3(like, k):
            kern = like.blocks["lh_grad_kernel"].kernel
            pv = like.param_vector("lh_grad_kernel", truth3)
            ob = L.c_buf()
            L.check(L.lib.mf_buffer_alloc(backend.handle, max(k, 1) * kern.nout * 8, C.byref(ob)))
            blk = like.blocks["lh_grad_kernel"].input

            def enq(count):
                ins = (L.c_buf * count)(*([blk.buf] * count))
                st = np.full(count, blk.stride, dtype=np.uint64)
                ns = np.full(count, n3, dtype=np.uint64)
                rows = np.ascontiguousarray(np.tile(pv, (count, 1)))
                u64p = C.POINTER(C.c_uint64)
                L.check(L.lib.mf_kernel_reduce_many(kern.handle, count, ins, st.ctypes.data_as(u64p),
                                                    ns.ctypes.data_as(u64p), L.dptr(rows), len(pv), ob))
            enq(3)
            backend.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            enq(k)
            e1.record(ext)
            e1.synchronize()
            L.lib.mf_buffer_free(ob)
            return e0.elapsed_time(e1) / 1e3 / k, kern.read_layout()["bytes_per_event"] * n3

        s32, b32 = timed3(l32, args.spwave_steps)
        s64, b64 = timed3(l64, max(20, args.spwave_steps // 4))
        f64_, g64_ = l64.likelihood_and_gradient(truth3)
        f32_, g32_ = l32.likelihood_and_gradient(truth3)
        hinv = np.linalg.inv(l64.hessian(truth3))
        sig = np.sqrt(2.0 * np.diag(hinv))
        spw = {"value": world / s32, "unit": "evals/s", "dtype": "f32 storage+arith, f64 sums",
               "config": f"K*mumu S+P wave with Legendre acceptance, 14 free parameters, {n3} events, mixed precision "
                         "(15 prepared columns folded from 17 hoisted)",
               "roofline": {"bound": "hbm", "achieved": b32 / s32 / 1e9, "peak": hbm_peak, "unit": "GB/s",
                            "frac": b32 / s32 / 1e9 / hbm_peak, "algorithmic_bytes_per_launch": b32},
               "f64": {"value": world / s64, "unit": "evals/s", "achieved_GBs": b64 / s64 / 1e9,
                       "algorithmic_bytes_per_launch": b64},
               "speedup_vs_f64": s64 / s32,
               "nll_abs_diff_vs_f64": abs(f32_ - f64_), "nll_rel_diff_vs_f64": abs(f32_ - f64_) / abs(f64_),
               "max_param_shift_sigma_vs_f64": float(np.max(np.abs(hinv @ (g32_ - g64_) / sig)))}
        del l32, l64

    # ---------------- batched toy study (4096 P-wave toys) ----------------
    toys = None
    if not args.no_toys:
        from morefit_gb300.toystudy import ToyStudy
        ts = ToyStudy(backend, spec, seed=229387429 + 1000 * rank)
        # warm-up: kernels compiled and cached, the segment schedule tuned for
        # the timed study's segment-size histogram (4096 toys of ~2000 events)
        ts.toy(4096, 2000, poisson=True, clip=(200, 50000), jitter=0.1)
        tuned = ts.tuning
        r = ts.toy(4096, 2000, poisson=True, clip=(200, 50000), jitter=0.1)
        serial = ts.serial_fits_per_s(r, 32)
        toys = {"value": world * 4096 / r.timing["total_s"], "unit": "toy fits/s",
                "fit_only": world * 4096 / r.timing["fit_s"],
                "serial_gpu_fits_per_s": serial,
                "batched_over_serial": (4096 / r.timing["fit_s"]) / serial,
                "config": "4096 K*mumu P-wave toys, Poisson(2000) events clipped to [200, 50000], each toy's "
                          "truth jittered by +-10% and used as its start; one GPU generation (one segment per toy) "
                          "+ precompute for all toys, batched Newton fits over ragged segments (F+grad, Hessian, "
                          "step trials per iteration)",
                "events": int(r.counts.sum()), "all_converged": bool(r.fit.converged.all()),
                "segment_schedule": str(ts.schedule),
                "schedule_reused": bool(ts.tuning and ts.tuning.get("cached")),
                "tuning_launch_ms": ({k: round(v * 1e3, 4) for k, v in tuned["launch_s"].items()}
                                     if tuned and "launch_s" in tuned else None),
                "max_iterations": int(r.fit.iterations.max()), "segment_launches": int(r.fit.evaluations),
                "pull_mean": [round(float(x), 3) for x in r.pulls.mean(0)],
                "pull_std": [round(float(x), 3) for x in r.pulls.std(0)]}

    # ---------------- serving loop: Poisson stream of fits, coalesced evaluations ----------------
    serving = None
    if not args.no_serving:
        from morefit_gb300.serving import FitServer, latency_summary, poisson_stream
        srv = FitServer(backend, hbm_budget=150 << 30, max_active=256)
        srv.run(poisson_stream(8, 1000.0, seed=3, nmax=20000), realtime=False)  # warm-up
        reqs = poisson_stream(args.serving_requests, args.serving_rate, seed=7 + rank)
        live = latency_summary(srv.run(reqs, realtime=True))
        cap = latency_summary(srv.run(reqs, realtime=False))
        ser = FitServer(backend, hbm_budget=150 << 30, max_active=1)
        ser.models = srv.models
        t0 = time.perf_counter()
        ser.run(reqs, realtime=False)
        serial = len(reqs) / (time.perf_counter() - t0)
        serving = {"value": live["fits_per_s"], "unit": "fits/s", "p50_ms": live["p50_ms"], "p99_ms": live["p99_ms"],
                   "config": f"{len(reqs)} fit requests, Poisson arrivals at {args.serving_rate:g}/s, 60% mass / 40% "
                             "S+P-wave fits, events log-uniform in [1k, 5M], FP32 per-event math with compensated "
                             "FP64 sums, HBM budget 150 GB; datasets generated on the device at admission",
                   "live": live, "capacity_all_at_once": cap, "serial_fits_per_s": serial,
                   "capacity_over_serial": cap["fits_per_s"] / serial}

    extras = None if args.no_extras else extra_rows(backend)
    fitters = None if args.no_fitters else fitter_rows(backend, host)

    # ---------------- CPU baseline (rank 0, N=1 only) ----------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import mforacle
        from oracle.spec_kernel import SpecKernel
        nthreads = os.cpu_count() or 1
        allc = cpu_reference_rate(host, nthreads, 1 << 30, args.cpu_seconds)
        one = cpu_reference_rate(host, 1, 1 << 30, args.cpu_seconds / 2)
        # configuration C1: the reference's mass lh_grad kernel text on 100k events, all host threads
        mspec = load_spec("mass")
        mk = {k["name"]: k for k in mspec["kernels"]}
        mev = generate_events(backend, mspec, 100_000, seed=229387429).download()
        mgk = SpecKernel(mk["lh_grad_kernel"])
        mlike = Likelihood(backend, mspec, np.float64)
        mpv = mlike.param_vector("lh_grad_kernel", mspec["truth"])
        mgk.reduce(mev, mpv, nthreads)
        t0 = time.perf_counter()
        mdone = 0
        while time.perf_counter() - t0 < 3.0:
            mgk.reduce(mev, mpv, nthreads)
            mdone += 1
        c1_cpu = {"value": mdone / (time.perf_counter() - t0), "unit": "evals/s", "cores": nthreads, "kind": "port",
                  "sample": f"{mdone} NLL+grad evaluations of the mass model over 100k events (~3 s)"}
        nll_gpu = -2.0 * float(like.sums("lh_grad_kernel", truth)[0])
        # the reference's whole fit (MIGRAD + HESSE) of dataset 0 on its CPU backend, one thread
        fit_1m = None
        kit = _refkit()
        if kit is not None:
            import tempfile
            with tempfile.TemporaryDirectory() as td:
                f0 = Path(td) / "pwave_1M.f64"
                np.ascontiguousarray(host).tofile(f0)
                fit_1m = _run_json([kit, "fitevents", "pwave", f0, 1])["fit_ms"]
        cpu = {"value": allc["value"], "unit": "evals/s", "cores": nthreads, "kind": allc["kind"],
               "sample": f"{allc['nevals']} NLL+grad evaluations over all {n} events of dataset 0 "
                         f"(~{args.cpu_seconds:g} s); {allc['how']}",
               "nthreads_1": {"value": one["value"], "unit": "evals/s", "cores": 1, "nevals": one["nevals"]},
               "events_fnv1a": mforacle.fnv1a(host),
               "nll_rel_diff_vs_gpu": abs(allc["nll"] - nll_gpu) / abs(nll_gpu), "c1_mass_100k": c1_cpu,
               "fit_1M_ms": fit_1m}

    if rank == 0:
        r3 = lambda x: None if x is None else float(f"{x:.4g}")
        # the targets' figures, last in the line so that a tail of the output shows them
        headline = {
            "fp64_evals_per_s": r3(value), "fp64_hbm_frac": r3(achieved / hbm_peak),
            "fp64_us_per_eval": r3(1e3 * ms64 / args.steps),
            "mixed_evals_per_s": r3(mixed["value"]) if mixed else None,
            "mixed_over_fp64": r3(mixed["speedup_vs_f64"]) if mixed else None,
            "mixed_nll_rel_diff": r3(mixed["nll_rel_diff_vs_f64"]) if mixed else None,
            "native_fp64_evals_per_s": r3(native["value"]) if native else None,
            "spwave_10M_mixed_evals_per_s": r3(spw["value"]) if spw else None,
            "spwave_10M_mixed_over_fp64": r3(spw["speedup_vs_f64"]) if spw else None,
            "spwave_10M_shift_sigma": r3(spw["max_param_shift_sigma_vs_f64"]) if spw else None,
            "toys_fits_per_s": r3(toys["value"]) if toys else None,
            "toys_fit_only_over_serial": r3(toys["batched_over_serial"]) if toys else None,
            "serving_fits_per_s": r3(serving["value"]) if serving else None,
            "serving_p50_ms": r3(serving["p50_ms"]) if serving else None,
            "serving_p99_ms": r3(serving["p99_ms"]) if serving else None,
            "serving_capacity_over_serial": r3(serving["capacity_over_serial"]) if serving else None,
            "e2e_evals_per_s": r3(world / e2e_s), "fit_loop_evals_per_s": r3(world / fit_loop_s),
            "reference_fitter_1M_fit_ms": r3(fitters["fit_1M"]["fit_ms"]) if fitters else None,
            "reference_fitter_fcn_grad_call_us":
                r3(fitters["fcn_call_us_1M"]["likelihood_and_gradient"]["p50"]) if fitters else None,
            "reference_fitter_threads_capacity_over_serial":
                r3(fitters["threads_8"]["capacity_over_serial"]) if fitters else None,
            "cpu_reference_1M_fit_ms": r3(cpu["fit_1M_ms"]) if cpu and cpu.get("fit_1M_ms") else None,
            "cpu_reference_evals_per_s": r3(cpu["value"]) if cpu else None,
            "cpu_reference_1thread_evals_per_s": r3(cpu["nthreads_1"]["value"]) if cpu else None}
        line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms64 / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64 (double-float arithmetic, 48-bit)",
                "data": "synthetic: seeded accept-reject K*mumu P-wave events generated on the GPU",
                "config": bench_config(n),
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                             "frac": achieved / hbm_peak, "traffic": NCU_TRAFFIC_F64,
                             "traffic_source": NCU_TRAFFIC_SOURCE, "peak_source": peak_kind,
                             "algorithmic_bytes_per_launch": bytes64},
                "e2e": {"value": world / e2e_s, "unit": "evals/s",
                        "h2d_bytes_per_step": int(host.nbytes), "d2h_bytes_per_step": nout * 8,
                        "what": "per step: raw events uploaded from page-locked host memory, precompute, prepare, "
                                f"NLL+grad, sums read to host; steps pipelined over {E2E_LANES} contexts",
                        "nll_rel_diff_vs_device": e2e_rel},
                "cpu_baseline": cpu,
                "clocks": clk.summary(),
                # K per-evaluation launches plus one combine per COMBINE_CHUNK
                "gpu_launches": args.steps + math.ceil(args.steps / COMBINE_CHUNK),
                "nll_truth": float(-2.0 * res64[0]),
                "e2e_mapped": {"value": world / e2e_mapped_s, "unit": "evals/s",
                               "h2d_bytes_per_step": int(host.nbytes), "d2h_bytes_per_step": nout * 8,
                               "nll_rel_diff_vs_device": e2e_mapped_rel},
                "e2e_sequential": {"value": world / seq_s, "unit": "evals/s",
                                   "h2d_bytes_per_step": int(host.nbytes), "d2h_bytes_per_step": nout * 8},
                "e2e_fit_loop": {"value": world / fit_loop_s, "unit": "evals/s", "h2d_bytes_per_step": 0,
                                 "d2h_bytes_per_step": nout * 8},
                "native_fp64": native, "mixed": mixed, "spwave_10M": spw, "toys": toys, "serving": serving,
                "extras": extras, "reference_fitter": fitters,
                "headline": headline}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


VARIANTS = {
    # name: (kernelT, native_f64, vec, block, bulk-copy pipeline, stages or unroll); 0 = library default
    "f64_native": (np.float64, True, 2, 256, False, 0),
    "f64_dw": (np.float64, False, 0, 0, False, 0),
    "f64_dw_b256": (np.float64, False, 1, 256, False, 0),
    "f64_dw_pipe": (np.float64, False, 1, 256, True, 4),
    "f64_dw_v2": (np.float64, False, 2, 256, False, 0),
    "f64_dw_u2": (np.float64, False, 2, 256, False, 2),
    "f64_dw_v1_u2": (np.float64, False, 1, 256, False, 2),
    "f64_dw_v2_u1": (np.float64, False, 2, 256, False, 1),
    "f64_dw_v1_u1": (np.float64, False, 1, 256, False, 1),
    "f64_dw_v1_b128": (np.float64, False, 1, 128, False, 0),
    "f64_dw_v1_b512": (np.float64, False, 1, 512, False, 0),
    "f32_u2": (np.float32, False, 4, 256, False, 2),
    "f32_v2_u2": (np.float32, False, 2, 256, False, 2),
    "f32_b512": (np.float32, False, 4, 512, False, 0),
    "f32_v2_b512_u2": (np.float32, False, 2, 512, False, 2),
    "f64_dw_v2_b512": (np.float64, False, 2, 512, False, 0),
    "f32": (np.float32, False, 0, 0, False, 0),
    "f32_v2": (np.float32, False, 2, 256, False, 0),
    "f32_pipe": (np.float32, False, 2, 256, True, 4),
}


def variants(args):
    """Times the NLL+grad kernel in each arithmetic mode / launch shape (one JSON line each).

    Same datasets and timing as the main benchmark; used for launch-shape
    sweeps and, with --steps 1, as the small case for ncu captures."""
    import ctypes as C
    import torch
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import CUDABackend
    from morefit_gb300.workloads import Likelihood, generate_events, load_spec
    torch.cuda.set_device(0)
    backend = CUDABackend(0, resident_idle_us=0)  # the launched kernels are the subject here
    spec = load_spec(args.model)
    kname = args.kernel
    truth = np.array(spec["truth"])
    n = args.nevents
    nsets = args.sets
    raw = [generate_events(backend, spec, n, seed=229387429 + r) for r in range(nsets)]
    ext = torch.cuda.ExternalStream(C_stream(backend))
    names = args.variant_list.split(",") if args.variant_list else list(VARIANTS)
    ref = None
    for name in names:
        kernelT, native, vec, block, pipeline, stages = VARIANTS[name]
        sets = []
        for r in range(nsets):
            like = Likelihood(backend, spec, kernelT, native_f64=native, vec=vec, block=block, pipeline=pipeline,
                              stages=stages)
            if kernelT == np.float64:
                like.set_device_data(raw[r])
            else:
                like.set_data(raw[r].download())
            sets.append(like)
        kern = sets[0].blocks[kname].kernel
        pv = sets[0].param_vector(kname, truth)
        K, W = args.steps, args.warmup
        out = L.c_buf()
        L.check(L.lib.mf_buffer_alloc(backend.handle, max(K, W, nsets, 1) * kern.nout * 8, C.byref(out)))

        def enqueue(count):
            ins = (L.c_buf * count)(*[sets[i % nsets].blocks[kname].input.buf for i in range(count)])
            st = np.array([sets[i % nsets].blocks[kname].input.stride for i in range(count)], np.uint64)
            ns = np.full(count, n, dtype=np.uint64)
            rows = np.ascontiguousarray(np.tile(pv, (count, 1)))
            u = C.POINTER(C.c_uint64)
            L.check(L.lib.mf_kernel_reduce_many(kern.handle, count, ins, st.ctypes.data_as(u), ns.ctypes.data_as(u),
                                                L.dptr(rows), len(pv), out))

        enqueue(nsets)  # untimed: makes every dataset's prepared columns
        if W:
            enqueue(W)
        backend.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        enqueue(K)
        e1.record(ext)
        e1.synchronize()
        backend.synchronize()
        ms = e0.elapsed_time(e1) / K
        res = np.zeros(kern.nout)
        L.check(L.lib.mf_buffer_d2h(out, 0, res.ctypes.data, kern.nout * 8))
        L.lib.mf_buffer_free(out)
        if ref is None:
            ref = res
        info = kern.info()
        bpe = kern.read_layout()["bytes_per_event"]
        row = {"variant": name, "us_per_eval": ms * 1e3, "evals_per_s": 1e3 / ms,
               "GBs": n * bpe / (ms * 1e-3) / 1e9, "bytes_per_event": bpe, "registers": info["registers"],
               "vec": info["vec"], "block": info["block"],
               "rel_diff_vs_first": (np.abs(res - ref) / np.maximum(np.abs(ref), 1.0)).max().item()}
        if args.lone:
            # synchronous single evaluations (Minuit2's call): mf_kernel_reduce
            # straight through ctypes, parameter vector and sums preallocated,
            # rotating over the datasets; host time per call
            sums = np.zeros(kern.nout)
            pvc = np.ascontiguousarray(pv)
            calls = [(sets[i].blocks[kname].input.buf, sets[i].blocks[kname].input.stride)
                     for i in range(nsets)]
            for i in range(min(20, args.lone_calls)):
                buf, st = calls[i % nsets]
                L.check(L.lib.mf_kernel_reduce(kern.handle, buf, st, n, L.dptr(pvc), len(pvc), L.dptr(sums)))
            host_us = []
            for i in range(args.lone_calls):
                buf, st = calls[i % nsets]
                t0 = time.perf_counter()
                L.check(L.lib.mf_kernel_reduce(kern.handle, buf, st, n, L.dptr(pvc), len(pvc), L.dptr(sums)))
                host_us.append((time.perf_counter() - t0) * 1e6)
            row["sync_call_us_median"] = statistics.median(host_us)
            row["sync_call_us_p10"] = sorted(host_us)[len(host_us) // 10]
        if args.lone_async:
            # single evaluations without the synchronous path's completion
            # signalling: mf_kernel_reduce_async (sums to device memory, no
            # system-scope fence or mapped-memory word), each followed by a
            # stream synchronize; the launch alone on the device, as ncu times it
            ob = L.c_buf()
            L.check(L.lib.mf_buffer_alloc(backend.handle, kern.nout * 8, C.byref(ob)))
            pvc = np.ascontiguousarray(pv)
            host_us = []
            for i in range(args.lone_calls):
                blk = sets[i % nsets].blocks[kname]
                t0 = time.perf_counter()
                L.check(L.lib.mf_kernel_reduce_async(kern.handle, blk.input.buf, blk.input.stride, n, L.dptr(pvc),
                                                     len(pvc), ob, 0))
                backend.synchronize()
                host_us.append((time.perf_counter() - t0) * 1e6)
            L.lib.mf_buffer_free(ob)
            row["async_call_us_median"] = statistics.median(host_us)
        print(json.dumps(row), flush=True)
        del sets


def _dropin():
    p = ROOT / "tests" / "cpp" / "_build" / platform.machine() / "dropin"
    return p if p.exists() else None


def _run_json(cmd, env=None):
    r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True, check=True, env=env)
    return json.loads(r.stdout.strip().splitlines()[-1])


def fitter_rows(backend, host):
    """The reference's own fitter + Minuit2 (MIGRAD + HESSE, analytic gradient
    and Hessian) over the C++ drop-in's CUDABlocks (tests/cpp/dropin, built
    where the reference sources are present): one fit of dataset 0 (1M P-wave
    events), and eight host threads each fitting a dataset of its own
    (20k-200k events) with their evaluations coalesced, against the same eight
    fits one after another. None where the drop-in is not built."""
    import tempfile
    from morefit_gb300.workloads import generate_events, load_spec
    d = _dropin()
    if d is None:
        return None
    spec = load_spec("pwave")
    out = {}
    with tempfile.TemporaryDirectory() as td:
        f0 = Path(td) / "pwave_1M.f64"
        np.ascontiguousarray(host).tofile(f0)
        fit = _run_json([d, "fit", "pwave", f0])
        out["fit_1M"] = {"fit_ms": fit["fit_ms"], "first_fit_ms": fit["first_fit_ms"], "cov_status": fit["cov_status"],
                         "events_fnv1a": fit["events_fnv1a"]}
        # one FCN evaluation as MIGRAD makes it (hoisted parameter buffers on
        # the host, CopyToParameterBuffer, SubmitKernel, Finish,
        # CopyFromKahanBuffer), per call, at the fitted point
        calls = _run_json([d, "calls", "pwave", f0, 2000])
        launch = _run_json([d, "calls", "pwave", f0, 2000, "launch"])
        calls_mixed = _run_json([d, "calls", "pwave", f0, 2000, "mixed"])
        out["fcn_call_us_1M"] = {"likelihood_and_gradient": calls["likelihood_and_gradient_us"],
                                 "likelihood": calls["likelihood_us"],
                                 "migrad_pattern_per_call": calls["migrad_pattern_us_per_call"],
                                 "resident_stats": calls["resident_stats"],
                                 "launch_per_call": {"likelihood_and_gradient": launch["likelihood_and_gradient_us"],
                                                     "likelihood": launch["likelihood_us"],
                                                     "migrad_pattern_per_call": launch["migrad_pattern_us_per_call"]},
                                 "mixed_likelihood_and_gradient": calls_mixed["likelihood_and_gradient_us"],
                                 "mixed_likelihood": calls_mixed["likelihood_us"]}
        files = []
        for i, n in enumerate([20000, 50000, 100000, 200000] * 2):
            p = Path(td) / f"pwave_{i}.f64"
            np.ascontiguousarray(generate_events(backend, spec, n, seed=1 + i).download()).tofile(p)
            files.append(p)
        mix = _run_json([d, "threads", "pwave", "coalesce", "f64", *files])
        serial = _run_json([d, "threads", "pwave", "serial", "f64", *files])
        plain = _run_json([d, "threads", "pwave", "plain", "f64", *files])
        lat = sorted(f["latency_ms"] for f in mix["fits"])
        out["threads_8"] = {"coalesced_ms": mix["wall_ms"], "serial_ms": serial["wall_ms"],
                            "threads_uncoalesced_ms": plain["wall_ms"],
                            "capacity_over_serial": serial["wall_ms"] / mix["wall_ms"],
                            "fit_latency_p50_ms": lat[len(lat) // 2], "fit_latency_max_ms": lat[-1],
                            "coalescer": mix["coalescer"],
                            "what": "8 host threads, each the reference's fitter + Minuit2 on its own P-wave dataset "
                                    "(20k-200k events) over its own CUDABackend, evaluations coalesced; against the "
                                    "same 8 fits one after another (kernel builds and uploads included)"}
    return out


def extra_rows(backend):
    """The rows around the headline path, each timed once on 1M events:
    weighted fit (Fisher kernel, corrected covariance), the Crystal Ball +
    polynomial model, one plot (integral kernel + GPU histogram + text), and
    event input from a file (page-cached .npy streamed to HBM)."""
    import ctypes as C
    import tempfile
    from morefit_gb300 import _lib as L
    from morefit_gb300.eventio import save_event_vector, upload_event_file
    from morefit_gb300.plotter import Plotter, PlotterOptions
    from morefit_gb300.workloads import Likelihood, generate_events, load_spec
    n = 1_000_000
    out = {}

    def rate(fn, k):
        fn()
        backend.synchronize()
        t0 = time.perf_counter()
        for _ in range(k):
            fn()
        return k / (time.perf_counter() - t0)

    # configuration C1: the 1D mass fit, 100k events, 4 parameters
    mass = load_spec("mass")
    c1 = generate_events(backend, mass, 100_000, seed=229387429)
    lm = Likelihood(backend, mass, np.float64)
    lm.set_device_data(c1)
    mlim = [(5200.0, 5400.0), (5.0, 50.0), (0.0, 1.0), (-0.01, 0.01)]
    lm.fit(limits=mlim)  # warm: kernels built
    t0 = time.perf_counter()
    rm = lm.fit(limits=mlim)
    c1_fit_ms = (time.perf_counter() - t0) * 1e3
    kern = lm.blocks["lh_grad_kernel"].kernel
    pv = lm.param_vector("lh_grad_kernel", mass["truth"])
    nb = 2000
    out_buf = L.c_buf()
    L.check(L.lib.mf_buffer_alloc(backend.handle, nb * kern.nout * 8, C.byref(out_buf)))
    inp = lm.blocks["lh_grad_kernel"].input
    ins = (L.c_buf * nb)(*([inp.buf] * nb))
    st = np.full(nb, inp.stride, dtype=np.uint64)
    ns = np.full(nb, 100_000, dtype=np.uint64)
    rows = np.ascontiguousarray(np.tile(pv, (nb, 1)))
    u64p = C.POINTER(C.c_uint64)

    def batch():
        L.check(L.lib.mf_kernel_reduce_many(kern.handle, nb, ins, st.ctypes.data_as(u64p), ns.ctypes.data_as(u64p),
                                            L.dptr(rows), len(pv), out_buf))
        backend.synchronize()
    batch()
    t0 = time.perf_counter()
    batch()
    batched = nb / (time.perf_counter() - t0)
    L.lib.mf_buffer_free(out_buf)
    out["c1_mass_100k"] = {
        "fit_ms": c1_fit_ms, "converged": bool(rm.converged[0]), "evaluations": int(rm.evaluations),
        "grad_evals_per_s": rate(lambda: lm.sums("lh_grad_kernel", mass["truth"]), 200),
        "batched_evals_per_s": batched,
        "what": "Gaussian + exponential mass fit, 100k events, FP64 (double-float), 4 parameters: damped Newton "
                "fit from the truth; synchronous evaluations; batched evaluations (2000 per call, one 0.8 MB "
                "dataset, L2-resident)"}

    # weighted mass fit: the mass events plus w_i = 0.5 + frac(i * 0.618...)
    mw = load_spec("mass_w")
    ev = generate_events(backend, load_spec("mass"), n, seed=11).download()
    f = np.arange(n, dtype=np.float64) * 0.6180339887498949
    evw = np.vstack([ev, 0.5 + (f - np.floor(f))])
    lw = Likelihood(backend, mw, np.float64)
    lw.set_data(evw)
    limits = [(5200.0, 5400.0), (5.0, 50.0), (0.0, 1.0), (-0.01, 0.01)]
    lw.fit(limits=limits)  # warm: kernels built
    t0 = time.perf_counter()
    r = lw.fit(limits=limits)
    fit_ms = (time.perf_counter() - t0) * 1e3
    out["weighted_mass_1M"] = {
        "fisher_evals_per_s": rate(lambda: lw.sums("lh_fisher_kernel", mw["truth"]), 200),
        "grad_evals_per_s": rate(lambda: lw.sums("lh_grad_kernel", mw["truth"]), 200),
        "fit_ms": fit_ms, "converged": bool(r.converged[0]), "evaluations": int(r.evaluations),
        "what": "synchronous evaluations (parameters in, sums out); fit = damped Newton from the truth + "
                "-2 H^-1 F H^-1 covariance"}
    # Crystal Ball + polynomial
    cb = load_spec("cbpoly")
    lc = Likelihood(backend, cb, np.float64)
    lc.set_device_data(generate_events(backend, cb, n, seed=12))
    cblim = [(-0.2, 0.4), (0.01, 0.2), (0.5, 5.0), (1.5, 10.0), (-1.0, 1.0), (-1.0, 1.0), (0.0, 1.0)]
    lc.fit(limits=cblim)  # warm: kernels built
    t0 = time.perf_counter()
    rc = lc.fit(limits=cblim)
    cb_fit_ms = (time.perf_counter() - t0) * 1e3
    out["cbpoly_1M"] = {"grad_evals_per_s": rate(lambda: lc.sums("lh_grad_kernel", cb["truth"]), 200),
                        "hessian_evals_per_s": rate(lambda: lc.sums("lh_hessian_kernel", cb["truth"]), 50),
                        "fit_ms": cb_fit_ms, "converged": bool(rc.converged[0]), "evaluations": int(rc.evaluations)}
    with tempfile.TemporaryDirectory() as td:
        # plot of the mass model over 1M device-resident events
        mass = load_spec("mass")
        cols = generate_events(backend, mass, n, seed=13)
        pl = Plotter(PlotterOptions(plotter="matplotlib", plot_pulls=True), backend)
        name = str(Path(td) / "mass_m.py")
        out["plot_mass_1M"] = {"plots_per_s": rate(lambda: pl.plot(mass, mass["truth"], cols, "m", name, 100), 20),
                               "what": "1000 integral bins (native FP64 kernel) + 100-bin GPU histogram + pulls + "
                                       "matplotlib text"}
        # event file: 10M P-wave events, 3 FP64 columns
        pw = load_spec("pwave")
        big = generate_events(backend, pw, 10 * n, seed=14).download()
        fpath = Path(td) / "pwave_10M.npy"
        save_event_vector(fpath, big)
        dims = pw["dimensions"]
        holder = {}

        def load():
            holder["c"] = upload_event_file(backend, fpath, dims)
        per_s = rate(load, 3)
        out["file_load_10M"] = {"GBs": big.nbytes * per_s / 1e9, "bytes": int(big.nbytes),
                                "what": "2-D SoA .npy (page cache warm) streamed through two 8 MiB page-locked "
                                        "chunks into HBM (mf_events_load_file)",
                                "exact": bool(np.array_equal(holder["c"].download()[:, :1000], big[:, :1000]))}
    return out


def C_stream(backend):
    import ctypes as C
    from morefit_gb300 import _lib as L
    p = C.c_void_p()
    L.check(L.lib.mf_context_stream(backend.handle, C.byref(p)))
    return p.value


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=25000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nevents", type=int, default=N_EVENTS)
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-toys", action="store_true")
    ap.add_argument("--no-spwave", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--serving-requests", type=int, default=200)
    ap.add_argument("--serving-rate", type=float, default=300.0)
    ap.add_argument("--spwave-events", type=int, default=10_000_000)
    ap.add_argument("--spwave-steps", type=int, default=400)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-native", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-fitters", action="store_true")
    ap.add_argument("--variants", action="store_true", help="time every kernel variant instead")
    ap.add_argument("--variant-list", default="")
    ap.add_argument("--sets", type=int, default=5)
    ap.add_argument("--lone", action="store_true", help="with --variants: also time synchronous single evaluations")
    ap.add_argument("--lone-calls", type=int, default=200)
    ap.add_argument("--lone-async", action="store_true",
                    help="with --variants: also time asynchronous single evaluations, one at a time")
    ap.add_argument("--model", default="pwave", help="with --variants: the model (a spec in morefit_gb300/specs)")
    ap.add_argument("--kernel", default="lh_grad_kernel", help="with --variants: the REDUCE kernel timed")
    args = ap.parse_args()
    if args.warmup < 3 and not args.variants:
        args.warmup = 3
    if args.impl == "reference":
        reference_arm(args)
    elif args.variants:
        variants(args)
    else:
        ours(args)


if __name__ == "__main__":
    main()
