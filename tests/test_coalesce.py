"""Many datasets per launch (mf_kernel_reduce_multi) and the coalescer of
concurrent host fitters (mf_coalescer_*), through the C ABI.

The reference evaluates one dataset per SubmitKernel and runs one fitter per
host thread (include/compute.hh:146, include/fitter.hh:113-169). The
multi-dataset launch evaluates many datasets in one launch; the coalescer
gathers the synchronous evaluations of several threads' contexts into such
launches. Both promise that a dataset's sums depend on nothing but its own
events and parameters: bit for bit the same alone and in any mix. Against
the single-dataset kernel (another summation order) they agree within the
FP64 bar the parity tests use (1e-12 of the sum of absolute values).
"""
import ctypes as C
import threading

import numpy as np
import pytest

SIZES = [1000, 5000, 100000, 1000000, 37, 4097]


def test_coalescer_needs_a_device():
    """Without a GPU, creating a coalescer fails cleanly (no dispatch thread left behind)."""
    from morefit_gb300 import _lib as L
    n = C.c_int(0)
    if L.lib.mf_device_count(C.byref(n)) == L.MF_OK and n.value > 0:
        pytest.skip("a device is visible")
    h = L.c_coal()
    assert L.lib.mf_coalescer_create(0, 0, 30, C.byref(h)) == L.MF_ERR_NO_DEVICE
    assert not h.value
    assert L.lib.mf_coalescer_destroy(None) == L.MF_OK


@pytest.fixture(scope="module")
def datasets():
    from morefit_gb300.backend import CUDABackend
    from morefit_gb300.workloads import Likelihood, generate_events, load_spec
    spec = load_spec("pwave")
    b = CUDABackend(0)
    likes = []
    for i, n in enumerate(SIZES):
        lk = Likelihood(b, spec, np.float64)
        lk.set_device_data(generate_events(b, spec, n, seed=1000 + i))
        likes.append(lk)
    yield spec, b, likes
    b.close()


def _multi(b, likes, idx, pv):
    from morefit_gb300 import _lib as L
    k = likes[0].blocks["lh_grad_kernel"].kernel
    cnt = len(idx)
    ins = (L.c_buf * cnt)(*[likes[i].blocks["lh_grad_kernel"].input.buf for i in idx])
    st = np.array([likes[i].blocks["lh_grad_kernel"].input.stride for i in idx], np.uint64)
    ns = np.array([SIZES[i] for i in idx], np.uint64)
    rows = np.ascontiguousarray(np.tile(pv, (cnt, 1)))
    ob = L.c_buf()
    L.check(L.lib.mf_buffer_alloc(b.handle, cnt * k.nout * 8, C.byref(ob)))
    u = C.POINTER(C.c_uint64)
    try:
        L.check(L.lib.mf_kernel_reduce_multi(k.handle, cnt, ins, st.ctypes.data_as(u), ns.ctypes.data_as(u),
                                             L.dptr(rows), len(pv), ob))
        out = np.zeros((cnt, k.nout))
        L.check(L.lib.mf_buffer_d2h(ob, 0, out.ctypes.data, out.nbytes))
    finally:
        L.lib.mf_buffer_free(ob)
    return out


@pytest.mark.gpu
def test_multi_dataset_launch(datasets, oracle_lib):
    spec, b, likes = datasets
    truth = np.array(spec["truth"])
    pv = likes[0].param_vector("lh_grad_kernel", truth)
    everything = _multi(b, likes, list(range(len(SIZES))), pv)
    for i in range(len(SIZES)):
        single = likes[i].sums("lh_grad_kernel", truth)
        # scale: the sums of |per-event terms| are below 50 x n for these outputs at the truth
        assert np.all(np.abs(everything[i] - single) <= 1e-10 * np.abs(single) + 1e-12 * 50 * SIZES[i]), i
        assert np.array_equal(_multi(b, likes, [i], pv)[0], everything[i]), f"dataset {i}: alone differs"
    # the same datasets in another order and with repeats: the same rows
    again = _multi(b, likes, [3, 0, 3, 5], pv)
    for row, i in zip(again, [3, 0, 3, 5]):
        assert np.array_equal(row, everything[i])


@pytest.mark.gpu
def test_coalescer_alone_and_in_the_mix():
    """Eight threads, each with its own context and dataset, evaluate NLL +
    gradient at 20 parameter points through one coalescer; every result
    equals the same evaluation made alone through the coalescer, and the
    single-dataset kernel's within the FP64 bar."""
    from morefit_gb300.backend import Coalescer, CUDABackend
    from morefit_gb300.workloads import Likelihood, generate_events, load_spec
    spec = load_spec("pwave")
    truth = np.array(spec["truth"])
    # near the truth: the accept-reject events have a positive density there
    thetas = [truth + 2e-4 * np.sin(np.arange(truth.size) + j) for j in range(20)]
    sizes = [2000, 50000, 300000, 1000, 2000, 50000, 300000, 1000]
    co = Coalescer(0, 0, 50)
    errors = []

    def worker(t, out, use):
        try:
            bb = CUDABackend(0)
            lk = Likelihood(bb, spec, np.float64)
            lk.set_device_data(generate_events(bb, spec, sizes[t], seed=77 + t))
            if use:
                bb.set_coalescer(co)
            out[t] = np.array([lk.sums("lh_grad_kernel", th) for th in thetas])
            bb.close()
        except Exception as e:  # reported below
            errors.append(repr(e))

    try:
        alone, plain = {}, {}
        for t in range(len(sizes)):
            worker(t, alone, True)
            worker(t, plain, False)
        mix = {}
        threads = [threading.Thread(target=worker, args=(t, mix, True)) for t in range(len(sizes))]
        for x in threads:
            x.start()
        for x in threads:
            x.join()
        assert not errors, errors
        for t in range(len(sizes)):
            assert np.all(np.isfinite(alone[t])), t
            assert np.array_equal(mix[t], alone[t]), f"thread {t}: in the mix differs from alone"
            tol = 1e-10 * np.abs(plain[t]) + 1e-12 * 50 * sizes[t]
            assert np.all(np.abs(mix[t] - plain[t]) <= tol), t
        st = co.stats()
        assert st["evaluations"] == 2 * len(sizes) * len(thetas)
        assert st["max_batch"] > 1, st
    finally:
        co.close()


@pytest.mark.gpu
def test_coalesced_submit_and_poll(datasets):
    """The asynchronous pair: tickets for several datasets, polled without and
    with waiting; each result equals the dataset's multi-dataset row."""
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import Coalescer
    spec, b, likes = datasets
    truth = np.array(spec["truth"])
    pv = likes[0].param_vector("lh_grad_kernel", truth)
    co = Coalescer(0, 0, 1000)
    try:
        tickets = []
        for i, lk in enumerate(likes):
            blk = lk.blocks["lh_grad_kernel"]
            t = C.c_uint64()
            L.check(L.lib.mf_coalesced_submit(co.handle, blk.kernel.handle, blk.input.buf, blk.input.stride, SIZES[i],
                                              L.dptr(pv), len(pv), C.byref(t)))
            tickets.append(t.value)
        out = np.zeros(likes[0].blocks["lh_grad_kernel"].kernel.nout)
        rc = L.lib.mf_coalesced_poll(co.handle, tickets[0], L.dptr(out), 0)
        assert rc in (L.MF_OK, L.MF_ERR_NOT_READY)
        if rc == L.MF_ERR_NOT_READY:
            L.check(L.lib.mf_coalesced_poll(co.handle, tickets[0], L.dptr(out), 1))
        got = [out.copy()]
        for t in tickets[1:]:
            L.check(L.lib.mf_coalesced_poll(co.handle, t, L.dptr(out), 1))
            got.append(out.copy())
        assert L.lib.mf_coalesced_poll(co.handle, tickets[0], L.dptr(out), 1) == L.MF_ERR_INVALID  # retired
        ref = _multi(b, likes, list(range(len(SIZES))), pv)
        for i in range(len(SIZES)):
            assert np.array_equal(got[i], ref[i]), i
    finally:
        co.close()
