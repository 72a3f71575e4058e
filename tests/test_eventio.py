"""On-disk event input (the reference's load_event_vector,
include/eventvector.hh:297-332, with NumPy files in place of a ROOT tree)."""
import numpy as np
import pytest


def _events(n=5000, seed=3):
    rng = np.random.default_rng(seed)
    return np.vstack([rng.uniform(-1, 1, n), rng.uniform(-1, 1, n), rng.uniform(-np.pi, np.pi, n)])


def test_formats_load_the_same_events(tmp_path):
    from morefit_gb300.eventio import load_event_vector, save_event_vector
    ev = _events()
    dims = ["ctl", "ctk", "phi"]
    save_event_vector(tmp_path / "soa.npy", ev)
    np.savez(tmp_path / "cols.npz", ctl=ev[0], ctk=ev[1], phi=ev[2], other=ev[0] * 2)
    rec = np.zeros(ev.shape[1], dtype=[("phi", "f8"), ("ctl", "f8"), ("ctk", "f8")])
    rec["ctl"], rec["ctk"], rec["phi"] = ev
    np.save(tmp_path / "rec.npy", rec)
    for f in ("soa.npy", "cols.npz", "rec.npy"):
        got = load_event_vector(tmp_path / f, dims)
        assert got.dtype == np.float64 and np.array_equal(got, ev), f
    # branch names differing from the dimension names, max_event
    got = load_event_vector(tmp_path / "cols.npz", ["a", "b"], branchnames=["phi", "other"], max_event=100)
    assert np.array_equal(got, np.vstack([ev[2, :100], 2 * ev[0, :100]]))
    got = load_event_vector(tmp_path / "soa.npy", ["x"], branchnames=["phi"], columns=dims)
    assert np.array_equal(got, ev[2:3])
    with pytest.raises(KeyError):
        load_event_vector(tmp_path / "cols.npz", ["m"])
    with pytest.raises(ValueError):
        load_event_vector(tmp_path / "cols.npz", ["ctl", "ctk"], branchnames=["ctl"])
    with pytest.raises(ValueError):
        load_event_vector(tmp_path / "soa.txt", dims)


@pytest.mark.gpu
def test_streamed_upload_matches_in_memory_upload(tmp_path, oracle_lib):
    """A 1M-event P-wave .npy streamed to the device equals the events, and
    the likelihood from it equals the one from the in-memory upload bit for
    bit; column subsets and order, FP32 storage, max_event, ragged chunks,
    FP32 files and a truncated file."""
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import CUDABackend
    from morefit_gb300.eventio import save_event_vector, upload_event_file
    from morefit_gb300.workloads import Likelihood, load_spec
    b = CUDABackend(0)
    try:
        ev = oracle_lib.generate("pwave", 1000003)  # more than one 8 MiB chunk per column
        dims = ["ctl", "ctk", "phi"]
        f = tmp_path / "pwave.npy"
        save_event_vector(f, ev)
        cols = upload_event_file(b, f, dims)
        assert np.array_equal(cols.download(), ev)
        spec = load_spec("pwave")
        a = Likelihood(b, spec, np.float64)
        a.set_device_data(cols)
        m = Likelihood(b, spec, np.float64)
        m.set_data(ev)
        th = spec["truth"]
        assert np.array_equal(a.sums("lh_grad_kernel", th), m.sums("lh_grad_kernel", th))
        sub = upload_event_file(b, f, ["x", "y"], branchnames=["phi", "ctl"], columns=dims, max_event=777)
        assert np.array_equal(sub.download(), ev[[2, 0], :777])
        f32 = upload_event_file(b, f, dims, elem=L.MF_F32)
        assert np.array_equal(f32.download(), ev.astype(np.float32))
        g = tmp_path / "pwave32.npy"
        save_event_vector(g, ev.astype(np.float32))
        assert np.array_equal(upload_event_file(b, g, dims).download(), ev.astype(np.float32).astype(np.float64))
        raw = f.read_bytes()
        (tmp_path / "short.npy").write_bytes(raw[:len(raw) // 2])
        with pytest.raises(L.MFError, match="too short"):
            upload_event_file(b, tmp_path / "short.npy", dims)
    finally:
        b.close()


@pytest.mark.gpu
def test_mapped_host_events_give_the_same_sums(oracle_lib):
    """Events read in place from host memory (mf_buffer_wrap_host: the
    precompute kernel, or for the mass model the column preparation, reads
    them over the host link) give the same sums, bit for bit, as events
    copied to HBM; plain (pageable) arrays are registered for the purpose."""
    from morefit_gb300.backend import CUDABackend
    from morefit_gb300.workloads import Likelihood, load_spec
    b = CUDABackend(0)
    try:
        for wl, n in (("pwave", 200000), ("mass", 100000)):
            ev = np.ascontiguousarray(oracle_lib.generate(wl, n))
            spec = load_spec(wl)
            a = Likelihood(b, spec, np.float64)
            a.set_data(ev)
            m = Likelihood(b, spec, np.float64)
            m.set_data_mapped(ev)
            b.synchronize()
            for kern in ("lh_kernel", "lh_grad_kernel"):
                assert np.array_equal(a.sums(kern, spec["truth"]), m.sums(kern, spec["truth"])), (wl, kern)
            # a second step over the same (re-written) host array
            ev[...] = oracle_lib.generate(wl, n, seed=4)
            m.set_data_mapped(ev)
            a.set_data(ev)
            b.synchronize()
            assert np.array_equal(a.sums("lh_grad_kernel", spec["truth"]), m.sums("lh_grad_kernel", spec["truth"]))
    finally:
        b.close()
