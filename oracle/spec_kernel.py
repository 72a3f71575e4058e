"""CPU oracle: the reference's kernel text, compiled with gcc (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the checker or the timed CPU baseline; the CUDA product
never does.

A kernel spec is what the reference's fitter hands to
ComputeBlock::MakeComputeKernel (include/fitter.hh:612-657): input column
names, parameter names and one ComputeGraphNode::get_kernel() string per
output, frozen as JSON under tests/golden/ by oracle/refkit. This module
wraps those strings in the same C loop as the reference's CPU backend
(include/compute_llvm.hh:535-750, restated in oracle/refkit/gcc_block.hh):
per event load every input column, evaluate every output, and add it to a
4-lane interleaved Kahan accumulator (lane = event % 4) whose lanes are
Kahan-combined at the end; with several threads, contiguous chunks of
n/nthreads events whose sums are Kahan-combined in chunk order
(compute_llvm.hh:751-932, utils.hh:14-26). Compiled with
``gcc -O3 -ffp-contract=off`` so the Kahan steps stay as written.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess
import tempfile
import threading
from pathlib import Path

import numpy as np

_CACHE = Path(os.environ.get("MOREFIT_ORACLE_CACHE", Path(tempfile.gettempdir()) / "morefit_oracle_kernels"))


def _c_source(name, inputs, params, exprs):
    M = len(exprs)
    L = []
    L.append("#include <math.h>\n")
    L.append(f"void {name}(unsigned nevents, unsigned from, unsigned to, const double* data, double* output,"
             " const double* parameters, double* kahan) {\n")
    for k, p in enumerate(params):
        L.append(f"  const double {p} = parameters[{k}];\n")
    L.append(f"  double lane_sum[{4 * M}], lane_c[{4 * M}];\n")
    L.append(f"  for (int q = 0; q < {4 * M}; q++) {{ lane_sum[q] = 0.0; lane_c[q] = 0.0; }}\n")
    L.append("  for (unsigned i = from; i < to; i++) {\n")
    for k, nm in enumerate(inputs):
        L.append(f"    const double {nm} = data[(unsigned long)nevents * {k}u + i];\n")
    for j, e in enumerate(exprs):
        L.append(f"    const double r{j} = {e};\n")
    L.append("    if (kahan) {\n      const unsigned lane = i % 4u;\n")
    for j in range(M):
        L.append(f"      {{ const unsigned q = {4 * j}u + lane; const double y = r{j} - lane_c[q];"
                 " const double t = lane_sum[q] + y; lane_c[q] = (t - lane_sum[q]) - y; lane_sum[q] = t; }\n")
    L.append("    } else {\n")
    for j in range(M):
        L.append(f"      output[(unsigned long)nevents * {j}u + i] = r{j};\n")
    L.append("    }\n  }\n")
    L.append(f"  if (kahan) {{\n    for (unsigned j = 0; j < {M}u; j++) {{\n"
             "      double s = 0.0, cc = 0.0;\n"
             "      for (unsigned l = 0; l < 4u; l++) { const double y = lane_sum[4u * j + l] - cc;"
             " const double t = s + y; cc = (t - s) - y; s = t; }\n"
             "      kahan[j] = s;\n    }\n  }\n}\n")
    return "".join(L)


def _kahan(values):
    s = 0.0
    c = 0.0
    for v in values:
        y = v - c
        t = s + y
        c = (t - s) - y
        s = t
    return s


class SpecKernel:
    """One compiled kernel spec. ``reduce`` mirrors a Kahan block, ``store`` a plain block."""

    _lock = threading.Lock()

    def __init__(self, spec: dict):
        self.name = spec["name"]
        self.inputs = list(spec["inputs"])
        self.params = list(spec["params"])
        self.exprs = list(spec["exprs"])
        src = _c_source(self.name, self.inputs, self.params, self.exprs)
        h = hashlib.sha256(src.encode()).hexdigest()[:20]
        so = _CACHE / f"{self.name}_{h}.so"
        with SpecKernel._lock:
            if not so.exists():
                _CACHE.mkdir(parents=True, exist_ok=True)
                c = _CACHE / f"{self.name}_{h}_{os.getpid()}.c"
                c.write_text(src)
                tmp = so.with_suffix(f".tmp{os.getpid()}.so")
                subprocess.run(["gcc", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(tmp), str(c), "-lm"],
                               check=True)
                os.replace(tmp, so)
                c.unlink(missing_ok=True)
        self._lib = C.CDLL(str(so))
        self._fn = getattr(self._lib, self.name)
        self._fn.restype = None
        self._fn.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]

    def _prep(self, events, params):
        ev = np.ascontiguousarray(events, dtype=np.float64)
        if ev.ndim == 1:
            ev = ev[None, :]
        if ev.shape[0] != len(self.inputs):
            raise ValueError(f"{self.name}: expected {len(self.inputs)} input columns, got {ev.shape[0]}")
        p = np.ascontiguousarray(params, dtype=np.float64)
        if p.size != len(self.params):
            raise ValueError(f"{self.name}: expected {len(self.params)} parameters, got {p.size}")
        return ev, (p if p.size else np.zeros(1))

    def reduce(self, events, params, nthreads: int = 1) -> np.ndarray:
        """Kahan sums of every output over all events (one list per call)."""
        ev, p = self._prep(events, params)
        n = ev.shape[1]
        M = len(self.exprs)
        nthreads = max(1, min(int(nthreads), max(1, n)))
        size = n // nthreads
        parts = np.zeros((nthreads, M))
        dummy = np.zeros(1)

        def run(t):
            frm = t * size
            to = n if t == nthreads - 1 else frm + size
            self._fn(n, frm, to, ev.ctypes.data, dummy.ctypes.data, p.ctypes.data, parts[t].ctypes.data)

        if nthreads == 1:
            run(0)
        else:
            ts = [threading.Thread(target=run, args=(t,)) for t in range(nthreads)]
            for t in ts:
                t.start()
            for t in ts:
                t.join()
        return np.array([_kahan(parts[:, j]) for j in range(M)])

    def store(self, events, params) -> np.ndarray:
        """Per-event outputs, shape (n_outputs, n)."""
        ev, p = self._prep(events, params)
        n = ev.shape[1]
        out = np.zeros((len(self.exprs), n))
        self._fn(n, 0, n, ev.ctypes.data, out.ctypes.data, p.ctypes.data, None)
        return out
