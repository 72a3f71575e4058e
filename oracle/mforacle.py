"""ctypes wrapper of the C oracle in oracle/mf_oracle.c (TEST INFRASTRUCTURE ONLY).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg only.
Build with ``make -C oracle port`` (``__graft_entry__.build()`` does it).
"""
from __future__ import annotations

import ctypes as C
import math
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libmforacle.so"
SEED = 229387429

MASS_TRUTH = [5280.0, 20.0, 0.3, -0.002]
MASS_RANGE = ([5000.0], [5600.0])
PWAVE_TRUTH = [0.70, -0.01, -0.15, -0.20, -0.10, 0.0, 0.0, 0.0]
PWAVE_RANGE = ([-1.0, -1.0, -math.pi], [1.0, 1.0, math.pi])


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        vp = C.c_void_p
        L.mfo_generate.argtypes = [C.c_int, vp, vp, vp, C.c_uint64, C.c_uint32, C.c_uint32, vp]
        L.mfo_generate.restype = C.c_int
        L.mfo_generate_partitioned.argtypes = [C.c_int, vp, vp, vp, C.c_uint64, C.c_uint32, C.c_uint32,
                                               C.c_uint32, vp]
        L.mfo_generate_partitioned.restype = C.c_int
        L.mfo_fnv1a.argtypes = [vp, C.c_uint64]
        L.mfo_fnv1a.restype = C.c_uint64
        L.mfo_pwave_basis.argtypes = [vp, C.c_uint32, vp]
        L.mfo_pwave_nll_grad.argtypes = [vp, C.c_uint32, vp, C.c_uint32, vp]
        L.mfo_mass_nll_grad.argtypes = [vp, C.c_uint32, vp, C.c_double, C.c_double, C.c_uint32, vp]
        L.mfo_seed_rows.argtypes = [C.c_uint64, C.c_uint32, vp]
        L.mfo_kahan.argtypes = [vp, C.c_uint32]
        L.mfo_kahan.restype = C.c_double
        L.mfo_pwave_max.argtypes = [vp]
        L.mfo_pwave_max.restype = C.c_double
        L.mfo_mass_max.argtypes = [vp, C.c_double, C.c_double]
        L.mfo_mass_max.restype = C.c_double
        _lib = L
    return _lib


def mass_weights(n: int) -> np.ndarray:
    """Event weights of the weighted mass workload, w_i = 0.5 + frac(i * 0.6180339887498949)
    (the column oracle/refkit appends after generation)."""
    f = np.arange(n, dtype=np.float64) * 0.6180339887498949
    return 0.5 + (f - np.floor(f))


def generate(workload: str, n: int, truth=None, seed: int = SEED, nthreads: int = 1) -> np.ndarray:
    """Seeded accept-reject events, shape (ndims, n), as the reference generates them
    (the weighted mass workload: the mass events plus the weight column)."""
    if workload == "mass_w":
        return np.vstack([generate("mass", n, truth, seed, nthreads), mass_weights(n)[None, :]])
    w = 0 if workload == "mass" else 1
    th = np.asarray(truth if truth is not None else (MASS_TRUTH if w == 0 else PWAVE_TRUTH), dtype=np.float64)
    lo, hi = (MASS_RANGE if w == 0 else PWAVE_RANGE)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    out = np.zeros((len(lo), n))
    rc = lib().mfo_generate(w, th.ctypes.data, lo.ctypes.data, hi.ctypes.data, seed, n, nthreads, out.ctypes.data)
    if rc:
        raise RuntimeError("mfo_generate failed")
    return out


def accelerator_partition(n: int, max_workitems: int = 8192):
    """(events per generator thread, generator threads) of the reference's
    accelerator generator for n events and compute_options::
    opencl_max_generator_workitems = max_workitems (compute_opencl.hh:437-445:
    nper = n / max + 1 when n exceeds max, else 1; thread t owns events
    [t * nper, (t + 1) * nper), so n / nper + 1 threads cover them)."""
    if max_workitems > 0 and n > max_workitems:
        nper = n // max_workitems + 1
        return nper, n // nper + 1
    return 1, max(n, 1)


def generate_partitioned(workload: str, n: int, nper: int, nseeds: int, truth=None, seed: int = SEED) -> np.ndarray:
    """Events with the accelerator partition: seed row t owns [t*nper, (t+1)*nper)."""
    w = 0 if workload == "mass" else 1
    th = np.asarray(truth if truth is not None else (MASS_TRUTH if w == 0 else PWAVE_TRUTH), dtype=np.float64)
    lo, hi = (MASS_RANGE if w == 0 else PWAVE_RANGE)
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    out = np.zeros((len(lo), n))
    if lib().mfo_generate_partitioned(w, th.ctypes.data, lo.ctypes.data, hi.ctypes.data, seed, n, nper, nseeds,
                                      out.ctypes.data):
        raise RuntimeError("mfo_generate_partitioned failed")
    return out


def fnv1a(a: np.ndarray) -> str:
    a = np.ascontiguousarray(a)
    return "%016x" % lib().mfo_fnv1a(a.ctypes.data, a.nbytes)


def seed_rows(nrows: int, seed: int = SEED) -> np.ndarray:
    out = np.zeros((4, nrows), dtype=np.uint32)
    lib().mfo_seed_rows(seed, nrows, out.ctypes.data)
    return out


def pwave_basis(events: np.ndarray) -> np.ndarray:
    ev = np.ascontiguousarray(events, dtype=np.float64)
    n = ev.shape[1]
    out = np.zeros((11, n))
    lib().mfo_pwave_basis(ev.ctypes.data, n, out.ctypes.data)
    return out


def pwave_nll_grad(basis: np.ndarray, theta, nthreads: int = 1) -> np.ndarray:
    b = np.ascontiguousarray(basis, dtype=np.float64)
    th = np.asarray(theta, dtype=np.float64)
    out = np.zeros(9)
    lib().mfo_pwave_nll_grad(b.ctypes.data, b.shape[1], th.ctypes.data, nthreads, out.ctypes.data)
    return out


def mass_nll_grad(m: np.ndarray, theta, nthreads: int = 1) -> np.ndarray:
    x = np.ascontiguousarray(m, dtype=np.float64).ravel()
    th = np.asarray(theta, dtype=np.float64)
    out = np.zeros(5)
    lib().mfo_mass_nll_grad(x.ctypes.data, x.size, th.ctypes.data, MASS_RANGE[0][0], MASS_RANGE[1][0], nthreads,
                            out.ctypes.data)
    return out
