"""Batched fits (ragged segments) and toy studies on the GPU.

The batched Newton fit is pinned to the reference's own fit of the same
events: MIGRAD + HESSE with analytic derivatives, run by the reference's
fitter in oracle/refkit (golden values and errors in tests/golden). Both
minimise the same -2 ln L; the reference stops at MIGRAD's EDM tolerance,
this fit at a Newton decrement of 1e-9, so values agree within a small
fraction of an error (bar: 0.05 sigma) and errors within 2e-3 relative.
"""
import numpy as np
import pytest

from conftest import golden_events, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from morefit_gb300.backend import CUDABackend
    b = CUDABackend(0)
    yield b
    b.close()


def _single_fit(backend, g, ev):
    from morefit_gb300.toystudy import PWAVE_LIMITS, SegmentLikelihood, fit_segments
    from morefit_gb300.workloads import Likelihood
    like = Likelihood(backend, g, np.float64)
    like.set_data(ev)
    sl = SegmentLikelihood(like, [0], [ev.shape[1]])
    return fit_segments(sl, np.array([g["truth"]]), PWAVE_LIMITS)


@pytest.mark.parametrize("n", [1000, 1000000])
def test_fit_matches_reference_migrad_hesse(backend, oracle_lib, n):
    g = load_golden(f"pwave_n{n}.json")
    ev = golden_events("pwave", n) if n == 1000 else oracle_lib.generate("pwave", n)
    if n != 1000:
        assert oracle_lib.fnv1a(ev) == g["events_fnv1a"]
    r = _single_fit(backend, g, ev)
    assert r.converged.all()
    ref_v = np.array(g["fit"]["values"])
    ref_e = np.array(g["fit"]["errors"])
    assert np.all(np.abs(r.values[0] - ref_v) <= 0.05 * ref_e), (r.values[0] - ref_v) / ref_e
    np.testing.assert_allclose(r.errors[0], ref_e, rtol=2e-3)


def test_batched_fits_equal_single_fits(backend):
    """A toy fitted among many gives the same result as fitted alone (one
    block per segment: the same arithmetic whatever the other segments)."""
    from morefit_gb300.toystudy import PWAVE_LIMITS, SegmentLikelihood, ToyStudy, fit_segments
    from morefit_gb300.workloads import load_spec
    spec = load_spec("pwave")
    ts = ToyStudy(backend, spec, seed=4242)
    res = ts.toy(64, 1500, poisson=True)
    assert res.fit.converged.all()
    like = None
    # refit toys 5 and 17 on their own, through the same event block
    from morefit_gb300.workloads import Likelihood, generate_events
    total = int(res.counts.sum())
    cols = generate_events(backend, spec, total, seed=4242, max_workitems=ts.generator_threads)
    like = Likelihood(backend, spec, np.float64)
    like.set_device_data(cols)
    begins = np.concatenate([[0], np.cumsum(res.counts)[:-1]])
    for t in (5, 17):
        sl = SegmentLikelihood(like, [begins[t]], [res.counts[t]])
        one = fit_segments(sl, res.truth[t:t + 1], PWAVE_LIMITS)
        assert np.array_equal(one.values[0], res.fit.values[t])
        assert np.array_equal(one.errors[0], res.fit.errors[t])


def test_toy_study_pulls_match_reference_toys(backend):
    """Config of the batched toy study: Poisson(2000) events clipped to
    [200, 50000], every toy's truth jittered by +-10%, each toy generated at
    and fitted from its own truth. The pull distributions of 2048 GPU toys
    match those of the 1000 toys run through the reference's own generator
    and fitter (MIGRAD + HESSE, tests/golden/toys_pwave_ref.json): per
    parameter, means within 3 combined standard errors and widths within 3
    combined standard errors of each other. The reference toys whose fit
    returned its start point (all pulls exactly 0: MIGRAD did not move, see
    test_fit_moves_where_the_reference_fit_stays) are left out; every GPU fit
    converges to a minimum."""
    from morefit_gb300.toystudy import ToyStudy
    from morefit_gb300.workloads import load_spec
    ref = load_golden("toys_pwave_ref.json")
    rp = np.array(ref["pulls"])
    assert ref["converged"] == ref["ntoys"]
    rp = rp[~np.all(rp == 0.0, axis=1)]
    res = ToyStudy(backend, load_spec("pwave"), seed=99).toy(2048, 2000, poisson=True, clip=(200, 50000),
                                                             jitter=0.1)
    assert res.fit.converged.all()
    assert res.counts.min() >= 200
    gp = res.pulls
    n_r, n_g = len(rp), len(gp)
    se_mean = 3.0 * np.sqrt(1.0 / n_r + 1.0 / n_g)
    se_std = 3.0 * np.sqrt(1.0 / (2 * n_r) + 1.0 / (2 * n_g))
    assert np.all(np.abs(gp.mean(0) - rp.mean(0)) < se_mean), (gp.mean(0), rp.mean(0))
    assert np.all(np.abs(gp.std(0) - rp.std(0)) < se_std), (gp.std(0), rp.std(0))


def test_segment_generation_is_independent_per_segment(backend):
    """Segment s's events depend only on its own streams, truth and bound:
    generating it alone gives the same events as within the batch."""
    from morefit_gb300.toystudy import generate_segments, pwave_maxprob
    from morefit_gb300.workloads import load_spec, splitmix_seed_rows
    spec = load_spec("pwave")
    rng = np.random.default_rng(5)
    truth = np.array(spec["truth"]) * (1.0 + rng.uniform(-0.1, 0.1, (5, 8)))
    counts = np.array([300, 1200, 17, 800, 2000])
    allv = generate_segments(backend, spec, truth, counts, pwave_maxprob(truth), seed=77, threads_per_seg=8).download()
    begins = np.concatenate([[0], np.cumsum(counts)[:-1]])
    assert np.all(np.abs(allv[:2]) <= 1.0) and np.all(np.abs(allv[2]) <= np.pi)
    # segment 3 alone, with its own seed rows (rows 24..31 of the batch's table)
    from morefit_gb300 import _lib as L
    import ctypes as C
    from morefit_gb300.backend import CUDABlock, DeviceColumns
    from morefit_gb300.toystudy import density_expression
    expr, params, bufs = density_expression(spec)
    gk = next(k for k in spec["kernels"] if k.get("generate"))
    blk = CUDABlock(backend, np.float64)
    blk.MakeGenerateKernel("g", 0, [], gk["outputs"], params, [expr], 1.0, ranges=list(zip(gk["lo"], gk["hi"])))
    from morefit_gb300.backend import eval_expressions_batch
    row = np.concatenate([truth[3:4], eval_expressions_batch(params[:8], truth[3:4], [e for _, e in bufs])], axis=1)
    seeds = np.ascontiguousarray(splitmix_seed_rows(40, 77)[:, 24:32], dtype=np.uint32)
    out = DeviceColumns(backend, L.MF_F64)
    out.ensure(3, int(counts[3]))
    L.check(L.lib.mf_kernel_generate_segments(
        blk.kernel.handle, seeds.ctypes.data_as(C.POINTER(C.c_uint32)), 8, 8, 1,
        np.array([0], np.uint64).ctypes.data_as(C.POINTER(C.c_uint64)),
        np.array([counts[3]], np.uint32).ctypes.data_as(C.POINTER(C.c_uint32)), L.dptr(np.ascontiguousarray(row)),
        row.shape[1], L.dptr(pwave_maxprob(truth[3:4])), out.buf, out.stride, 10000000))
    alone = out.download()
    assert np.array_equal(alone, allv[:, begins[3]:begins[3] + counts[3]])


def test_fit_moves_where_the_reference_fit_stays(backend):
    """Toy datasets on which the reference's MIGRAD returns its start point
    (tests/golden/toys_pwave_stuck.json): this fit, from the same start,
    converges to a point with a lower -2 ln L and a vanishing gradient."""
    from pathlib import Path
    from morefit_gb300.toystudy import PWAVE_LIMITS
    from morefit_gb300.workloads import Likelihood, load_spec
    g = load_golden("toys_pwave_stuck.json")
    ev = np.fromfile(Path(__file__).parent / "golden" / "toys_pwave_stuck_events.f64").reshape(3, -1)
    begins = np.concatenate([[0], np.cumsum(g["counts"])[:-1]])
    spec = load_spec("pwave")
    for k, n in enumerate(g["counts"]):
        like = Likelihood(backend, spec, np.float64)
        like.set_data(np.ascontiguousarray(ev[:, begins[k]:begins[k] + n]))
        r = like.fit(g["truths"][k], limits=PWAVE_LIMITS)
        assert r.converged[0]
        f_start, _ = like.likelihood_and_gradient(g["ref_values"][k])
        f_min, grad = like.likelihood_and_gradient(r.values[0])
        assert f_min < f_start - 1.0, (f_min, f_start)
        assert np.abs(grad).max() < 1e-3, grad


def test_segment_schedule_tuned_and_reused(backend, tmp_path, monkeypatch):
    """The toy study's tuner measures every candidate schedule of the segment
    kernels (threads per block; one block per segment, or runs of block x
    2..16 events per block combined per segment), keeps the fastest, and a
    later study of the same model and segment-size histogram reuses it
    without measuring: from the process's table, and in a process whose
    table is empty from the MOREFIT_GB300_CACHE file. Fits run with the
    chosen schedule converge, and a toy fitted alone with it gives the
    batch's result bit for bit."""
    from morefit_gb300 import toystudy as T
    from morefit_gb300.workloads import load_spec
    monkeypatch.setenv("MOREFIT_GB300_CACHE", str(tmp_path))
    monkeypatch.setattr(T, "_SCHEDULES", {})
    spec = load_spec("pwave")
    cfg = dict(poisson=True, clip=(200, 50000), jitter=0.1)
    a = T.ToyStudy(backend, spec, seed=11)
    ra = a.toy(512, 2000, **cfg)
    assert a.tuning is not None and not a.tuning["cached"]
    times = a.tuning["launch_s"]
    cands = a.candidates(ra.counts)
    assert len(times) == len(cands) and any(c.events_per_block for c in cands)
    assert str(a.schedule) == min(times, key=times.get)
    assert ra.fit.converged.all()
    print("segment schedules (ms per Newton iteration's launches):",
          {k: round(v * 1e3, 3) for k, v in sorted(times.items(), key=lambda kv: kv[1])})
    assert (tmp_path / "toy_schedules.json").exists()

    b = T.ToyStudy(backend, spec, seed=12)
    rb = b.toy(512, 2000, **cfg)
    assert b.tuning["cached"] and b.schedule == a.schedule and "launch_s" not in b.tuning
    assert rb.fit.converged.all()

    monkeypatch.setattr(T, "_SCHEDULES", {})  # another process: the file only
    c = T.ToyStudy(backend, spec, seed=11)
    rc = c.toy(512, 2000, **cfg)
    assert c.tuning["cached"] and c.schedule == a.schedule
    assert np.array_equal(rc.fit.values, ra.fit.values)

    # a toy alone under the chosen schedule
    t = 7
    sl = c._last_segments
    one = T.SegmentLikelihood(sl.like, sl.begins[t:t + 1], sl.counts[t:t + 1], c.schedule.events_per_block)
    r1 = T.fit_segments(one, rc.truth[t:t + 1], c.limits)
    assert np.array_equal(r1.values[0], rc.fit.values[t])
