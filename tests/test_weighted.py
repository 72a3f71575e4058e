"""Weighted fits on the GPU: the Fisher kernel and the covariance correction.

Weighted mass workload: the Gaussian + exponential mass model with an event
weight column w_i = 0.5 + frac(i * 0.6180339887498949); the reference
multiplies log p by w (fitter.hh:337-338), adds the Fisher kernel
d(w log p)/dtheta_i * d(w log p)/dtheta_j (fitter.hh:471-523) and reports
errors from -2 H^-1 F H^-1 (fitter.hh:894-994). Golden sums, matrices and the
reference's fit (MIGRAD + HESSE + correction) come from oracle/refkit.
Bars as in the other parity tests: FP64 sums within 1e-10 relative (1e-12 of
the sum of absolute per-event terms); fitted values within 0.05 sigma and
corrected errors within 2e-3 relative of the reference's.
"""
import numpy as np
import pytest

from conftest import assert_sums_close, golden_events, kernel_spec, load_golden
from oracle.spec_kernel import SpecKernel

pytestmark = pytest.mark.gpu

KERNELS = ("lh_kernel", "lh_grad_kernel", "lh_hessian_kernel", "lh_fisher_kernel")
MASS_LIMITS = [(5200.0, 5400.0), (5.0, 50.0), (0.0, 1.0), (-0.01, 0.01)]


@pytest.fixture(scope="module")
def backend():
    from morefit_gb300.backend import CUDABackend
    b = CUDABackend(0)
    yield b
    b.close()


def _events(oracle_lib, n):
    g = load_golden(f"mass_w_n{n}.json")
    ev = golden_events("mass_w", n) if n == 1000 else oracle_lib.generate("mass_w", n)
    assert oracle_lib.fnv1a(ev) == g["events_fnv1a"]
    return g, ev


@pytest.mark.parametrize("native", [False, True])
@pytest.mark.parametrize("n", [1000, 100000])
def test_weighted_sums_match_reference_golden(backend, oracle_lib, n, native):
    from morefit_gb300.workloads import Likelihood
    g, ev = _events(oracle_lib, n)
    like = Likelihood(backend, g, np.float64, native_f64=native)
    like.set_data(ev)
    for pt in g["points"]:
        for name in KERNELS:
            p = pt["kernel_params"][name]
            got = like.sums(name, param_vector=p)
            ref = np.array(pt["kernel_sums"][name])
            scale = np.abs(SpecKernel(kernel_spec(g, name)).store(ev, p)).sum(axis=1)
            assert_sums_close(got, ref, scale, what=f"mass_w n={n} {name}")


def test_fisher_matrix_as_the_fitter_returns_it(backend, oracle_lib):
    from morefit_gb300.workloads import Likelihood
    g, ev = _events(oracle_lib, 1000)
    like = Likelihood(backend, g, np.float64)
    like.set_data(ev)
    for pt in g["points"]:
        f = like.fisher(pt["params"])
        np.testing.assert_allclose(f.ravel(), pt["fisher"], rtol=1e-9, atol=1e-10 * np.abs(pt["fisher"]).max())
        assert np.allclose(f, f.T)


def test_weighted_fit_matches_reference(backend, oracle_lib):
    """Fit of 100k weighted events from the truth: values and corrected
    errors against the reference's MIGRAD + HESSE + correction."""
    from morefit_gb300.workloads import Likelihood
    g, ev = _events(oracle_lib, 100000)
    like = Likelihood(backend, g, np.float64)
    like.set_data(ev)
    r = like.fit(limits=MASS_LIMITS)
    assert r.converged[0]
    ref_v = np.array(g["fit"]["values"])
    ref_e = np.array(g["fit"]["errors"])
    assert np.all(np.abs(r.values[0] - ref_v) <= 0.05 * ref_e), (r.values[0] - ref_v) / ref_e
    np.testing.assert_allclose(r.errors[0], ref_e, rtol=2e-3)


def test_unweighted_model_has_no_fisher_kernel(backend):
    from morefit_gb300.workloads import Likelihood
    g = load_golden("mass_n1000.json")
    like = Likelihood(backend, g, np.float64)
    like.set_data(golden_events("mass", 1000))
    with pytest.raises(ValueError):
        like.fisher(g["truth"])


def test_weighted_mixed_precision_shift(backend, oracle_lib):
    """FP32 arithmetic over the FP64 columns moves the weighted estimate by at
    most 1e-3 of its corrected error: dtheta = -H^-1 (g32 - g64)."""
    from morefit_gb300.workloads import Likelihood, weighted_covariance
    g, ev = _events(oracle_lib, 100000)
    l64 = Likelihood(backend, g, np.float64)
    l64.set_data(ev)
    l32 = Likelihood(backend, g, np.float32)
    l32.set_data(ev)
    for pt in g["points"]:
        th = pt["params"]
        f64, g64 = l64.likelihood_and_gradient(th)
        f32, g32 = l32.likelihood_and_gradient(th)
        h = l64.hessian(th)
        sigma = np.sqrt(np.diag(weighted_covariance(h, l64.fisher(th))))
        shift = -np.linalg.solve(h, g32 - g64) / sigma
        assert np.abs(shift).max() <= 1e-3, shift
        assert abs(f32 - f64) <= 1e-6 * abs(f64)
