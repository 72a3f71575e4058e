"""Resident evaluations (mf_context_set_resident) on the GPU.

A context watches its synchronous REDUCE calls, builds a module with the per-
block work of its two most used kernels and then serves their evaluations
from one grid that stays on the device and waits for requests in mapped host
memory. Each request runs the kernel's own block partition and combine, so
the sums must equal a launch's bit for bit; the grid must leave when idle and
make room when anything else is launched on the device.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _warm(backend, like, theta, timeout=120.0):
    t0 = time.time()
    while backend.resident_stats()["state"] < 2 and time.time() - t0 < timeout:
        like.sums("lh_grad_kernel", theta)
        like.sums("lh_kernel", theta)
    assert backend.resident_stats()["state"] == 2, backend.resident_stats()


def _pair(spec, kernelT, n, seed=11, idle_us=2000):
    from morefit_gb300.backend import CUDABackend
    from morefit_gb300.workloads import Likelihood, generate_events
    out = []
    for idle in (0, idle_us):
        b = CUDABackend(0, resident_idle_us=idle)
        lk = Likelihood(b, spec, kernelT)
        lk.set_device_data(generate_events(b, spec, n, seed=seed))
        out.append((b, lk))
    return out


@pytest.mark.parametrize("workload,kernelT,n", [("pwave", np.float64, 1000000), ("pwave", np.float32, 100000),
                                                ("mass", np.float64, 100000), ("spwave", np.float64, 20000),
                                                ("pwave", np.float64, 37)])
def test_resident_sums_equal_launches(workload, kernelT, n):
    """MIGRAD's pattern (a gradient, then two values) at 30 points: every sum
    served by the resident grid equals the launched one bit for bit."""
    from morefit_gb300.workloads import load_spec
    spec = load_spec(workload)
    truth = np.array(spec["truth"])
    # idle time far above any pause between the calls below (a garbage
    # collection, a busy host): every call is served by the same grid
    (b0, l0), (b1, l1) = _pair(spec, kernelT, n, idle_us=500000)
    calls = [(kern, truth * (1.0 + 1e-3 * np.sin(np.arange(truth.size) + j)))
             for j in range(30) for kern in ("lh_grad_kernel", "lh_kernel", "lh_kernel")]
    try:
        launched = [l0.sums(kern, th).copy() for kern, th in calls]  # sums() returns a reused array
        _warm(b1, l1, truth)
        time.sleep(0.03)  # past the hold after the other context's launches
        l1.sums("lh_kernel", truth)  # starts the grid if none is up
        before = b1.resident_stats()["served"]
        served = [l1.sums(kern, th).copy() for kern, th in calls]
        st = b1.resident_stats()
        # every call served by the grid (no other launch on the device meanwhile)
        assert st["served"] - before == len(calls), st
        assert st["blocks"] > 0 and st["grids"] >= 1
        for (kern, _), a, b in zip(calls, launched, served):
            assert np.array_equal(a, b), (kern, a, b)
    finally:
        del l0, l1
        b0.close()
        b1.close()


def test_resident_grid_makes_room_and_leaves_when_idle():
    """Another context's launch on the device asks the grid to leave, and that
    launch completes promptly; the grid comes back after the hold. Idle for
    longer than idle_us, the grid leaves by itself and a later call starts a
    new one. Every sum equals the launched one."""
    from morefit_gb300.backend import CUDABackend
    from morefit_gb300.workloads import generate_events, load_spec
    spec = load_spec("pwave")
    truth = np.array(spec["truth"])
    # idle_us 50 ms: above any host pause between back-to-back calls, below the sleeps
    (b0, l0), (b1, l1) = _pair(spec, np.float64, 200000, idle_us=50000)
    other = CUDABackend(0, resident_idle_us=0)
    try:
        ref = l0.sums("lh_grad_kernel", truth)
        _warm(b1, l1, truth)
        time.sleep(0.03)  # past the hold after the other context's launches
        l1.sums("lh_kernel", truth)  # starts the grid if none is up
        s0 = b1.resident_stats()
        for _ in range(3):
            assert np.array_equal(l1.sums("lh_grad_kernel", truth), ref)
        s1 = b1.resident_stats()
        assert s1["served"] == s0["served"] + 3, (s0, s1)
        # another context launches while the grid is up: its work is not held back
        t0 = time.perf_counter()
        ev = generate_events(other, spec, 10000, seed=3)
        other.synchronize()
        assert time.perf_counter() - t0 < 1.0
        assert np.array_equal(l1.sums("lh_grad_kernel", truth), ref)
        time.sleep(0.03)  # past the hold: the calls after the next start a new grid
        for _ in range(4):
            assert np.array_equal(l1.sums("lh_grad_kernel", truth), ref)
        s2 = b1.resident_stats()
        assert s2["grids"] > s1["grids"] and s2["served"] > s1["served"], (s1, s2)
        # idle for longer than idle_us: the grid leaves by itself
        time.sleep(0.1)
        for _ in range(3):
            assert np.array_equal(l1.sums("lh_grad_kernel", truth), ref)
        s3 = b1.resident_stats()
        assert s3["grids"] > s2["grids"], (s2, s3)
        del ev
    finally:
        del l0, l1
        other.close()
        b0.close()
        b1.close()
