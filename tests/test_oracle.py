"""The oracle against the reference's own outputs (CPU only).

Golden files were written by oracle/refkit: the reference's generator,
fitter and Minuit2 running on the reference's kernel text (make_golden.sh).
"""
from pathlib import Path

import numpy as np
import pytest

from conftest import assert_sums_close, golden_events, kernel_spec, load_golden
from oracle.spec_kernel import SpecKernel


@pytest.mark.parametrize("workload,n", [("pwave", 1000), ("mass", 1000), ("mass_w", 1000)])
def test_generator_reproduces_reference_events(oracle_lib, workload, n):
    ev = oracle_lib.generate(workload, n)
    ref = golden_events(workload, n)
    assert np.array_equal(ev, ref)
    assert oracle_lib.fnv1a(ev) == load_golden(f"{workload}_n{n}.json")["events_fnv1a"]


@pytest.mark.parametrize("workload,n", [("mass", 100000), ("mass_w", 100000), ("pwave", 1000000)])
def test_generator_hash_at_full_size(oracle_lib, workload, n):
    ev = oracle_lib.generate(workload, n)
    assert oracle_lib.fnv1a(ev) == load_golden(f"{workload}_n{n}.json")["events_fnv1a"]


def test_generator_threads_partition(oracle_lib):
    # Per-thread streams (generator.hh:102-113): thread t starts from t jumps.
    a = oracle_lib.generate("pwave", 4000, nthreads=4)
    b = oracle_lib.generate("pwave", 4000, nthreads=1)
    assert np.array_equal(a[:, :1000], b[:, :1000])
    assert not np.array_equal(a[:, 1000:2000], b[:, 1000:2000])


def _inputs_for(g, events, spec_name):
    """Event block a kernel reads: raw events, or the precompute output."""
    ks = {k["name"]: k for k in g["kernels"]}
    if "precompute_kernel" in ks:
        return SpecKernel(ks["precompute_kernel"]).store(events, [])
    return events


@pytest.mark.parametrize("workload,n", [("pwave", 1000), ("mass", 1000), ("mass_w", 1000), ("cbpoly", 1000),
                                        ("spwave", 2000)])
def test_spec_kernel_reproduces_reference_sums(oracle_lib, workload, n):
    g = load_golden(f"{workload}_n{n}.json")
    ev = golden_events(workload, n)
    names = [k["name"] for k in g["kernels"] if k["name"].startswith("lh_")]
    assert ("lh_fisher_kernel" in names) == (workload == "mass_w")
    for name in names:
        sk = SpecKernel(kernel_spec(g, name))
        cols = _inputs_for(g, ev, name)
        for pt in g["points"]:
            got = sk.reduce(cols, pt["kernel_params"][name])
            ref = np.array(pt["kernel_sums"][name])
            np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())


def test_spec_kernel_threads(oracle_lib):
    g = load_golden("pwave_n1000.json")
    ev = golden_events("pwave", 1000)
    sk = SpecKernel(kernel_spec(g, "lh_grad_kernel"))
    cols = _inputs_for(g, ev, "lh_grad_kernel")
    p = g["points"][0]["kernel_params"]["lh_grad_kernel"]
    a = sk.reduce(cols, p, nthreads=1)
    b = sk.reduce(cols, p, nthreads=7)
    np.testing.assert_allclose(a, b, rtol=1e-14, atol=1e-12)


def test_closed_form_pwave_matches_reference(oracle_lib):
    g = load_golden("pwave_n1000.json")
    ev = golden_events("pwave", 1000)
    basis = oracle_lib.pwave_basis(ev)
    for pt in g["points"]:
        got = oracle_lib.pwave_nll_grad(basis, pt["params"])
        ref = np.array(pt["kernel_sums"]["lh_grad_kernel"])
        assert_sums_close(got, ref, np.abs(ref) + 1e3, rtol=1e-11, stol=1e-13, what="pwave closed form")


def test_closed_form_mass_matches_reference(oracle_lib):
    g = load_golden("mass_n1000.json")
    ev = golden_events("mass", 1000)
    for pt in g["points"]:
        got = oracle_lib.mass_nll_grad(ev[0], pt["params"])
        ref = np.array(pt["kernel_sums"]["lh_grad_kernel"])
        assert_sums_close(got, ref, np.abs(ref) + 1e3, rtol=1e-9, stol=1e-12, what="mass closed form")


def test_closed_form_pwave_full_size(oracle_lib):
    g = load_golden("pwave_n1000000.json")
    ev = oracle_lib.generate("pwave", 1000000, nthreads=1)
    basis = oracle_lib.pwave_basis(ev)
    pt = g["points"][0]
    got = oracle_lib.pwave_nll_grad(basis, pt["params"], nthreads=4)
    ref = np.array(pt["kernel_sums"]["lh_grad_kernel"])
    assert_sums_close(got, ref, np.full(9, 1e6), rtol=1e-11, stol=1e-13, what="pwave 1M closed form")


@pytest.mark.parametrize("n", [1000, 100000])
def test_weighted_covariance_reproduces_reference_errors(n):
    """The reference's weighted fit reports sqrt(diag(-2 H^-1 F H^-1)) at its
    minimum (fitter.hh:894-994); H and F at that point are in the golden file."""
    from morefit_gb300.workloads import weighted_covariance
    g = load_golden(f"mass_w_n{n}.json")
    pt = g["points"][1]
    assert pt["params"] == g["fit"]["values"]
    npar = len(g["parameters"])
    cov = weighted_covariance(np.reshape(pt["hessian"], (npar, npar)), np.reshape(pt["fisher"], (npar, npar)))
    np.testing.assert_allclose(np.sqrt(np.diag(cov)), g["fit"]["errors"], rtol=1e-9)
    # the correction is not the unweighted 2 H^-1
    plain = np.sqrt(np.diag(2.0 * np.linalg.inv(np.reshape(pt["hessian"], (npar, npar)))))
    assert np.abs(plain / np.array(g["fit"]["errors"]) - 1.0).max() > 0.01


def test_reference_fitter_returns_the_start_point_on_some_toys(oracle_lib):
    """On these P-wave toy datasets (tests/golden/make_stuck_toys.py) the
    reference's fitter, started at the truth, returns the truth unmoved and
    reports success; the gradient of -2 ln L there is far from zero, so the
    point is not a minimum. About one toy in ten behaves so (74 of the 1000
    reference toys in toys_pwave_ref.json have all pulls exactly 0)."""
    g = load_golden("toys_pwave_stuck.json")
    raw = np.fromfile(Path(__file__).parent / "golden" / "toys_pwave_stuck_events.f64")
    ev = raw.reshape(3, -1)
    begins = np.concatenate([[0], np.cumsum(g["counts"])[:-1]])
    for k, n in enumerate(g["counts"]):
        assert g["ref_values"][k] == g["truths"][k]
        basis = oracle_lib.pwave_basis(ev[:, begins[k]:begins[k] + n])
        grad = -2.0 * oracle_lib.pwave_nll_grad(basis, np.array(g["truths"][k]))[1:]
        assert np.abs(grad).max() > 50.0, grad
    ref = np.array(load_golden("toys_pwave_ref.json")["pulls"])
    assert 0.03 < np.all(ref == 0.0, axis=1).mean() < 0.15
