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
        one = fit_segments(sl, np.array([res.truth]), PWAVE_LIMITS)
        assert np.array_equal(one.values[0], res.fit.values[t])
        assert np.array_equal(one.errors[0], res.fit.errors[t])


def test_toy_study_pulls(backend):
    """256 toys of Poisson(2000) events: every fit converges and the pulls of
    every parameter have mean within 0.35 of 0 and width within 0.15 of 1
    (seeded, so the outcome is fixed). The mean bar leaves room for the
    maximum-likelihood estimator's finite-sample bias: S4's pull mean is
    -0.20 +- 0.02 over 4096 such toys."""
    from morefit_gb300.toystudy import ToyStudy
    from morefit_gb300.workloads import load_spec
    res = ToyStudy(backend, load_spec("pwave"), seed=99).toy(256, 2000, poisson=True, clip=(200, 50000))
    assert res.fit.converged.all()
    assert res.counts.min() >= 200
    mean = res.pulls.mean(axis=0)
    std = res.pulls.std(axis=0)
    assert np.all(np.abs(mean) < 0.35), mean
    assert np.all(np.abs(std - 1.0) < 0.15), std
