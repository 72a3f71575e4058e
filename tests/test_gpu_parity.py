"""CUDA backend against the reference's own numbers (GB300).

Golden sums come from the reference's fitter on the reference's kernel text
(tests/golden, oracle/refkit); edge cases and large sizes are checked against
the same kernel text compiled for the CPU (oracle/spec_kernel.py) or the C
restatement (oracle/mf_oracle.c). Bars: FP64 within 1e-10 relative on the NLL
(and, for gradient/Hessian sums that can be near zero, within 1e-12 of the
sum of absolute per-event terms); mixed precision within 2e-6 of that sum.
"""
import numpy as np
import pytest

from conftest import assert_sums_close, golden_events, kernel_spec, load_golden
from oracle.spec_kernel import SpecKernel

pytestmark = pytest.mark.gpu

KERNELS = ("lh_kernel", "lh_grad_kernel", "lh_hessian_kernel")


@pytest.fixture(scope="module")
def backend():
    from morefit_gb300.backend import CUDABackend
    b = CUDABackend(0)
    yield b
    b.close()


def _abs_scale(g, name, cols, params):
    per_event = SpecKernel(kernel_spec(g, name)).store(cols, params)
    return np.abs(per_event).sum(axis=1)


def _cols(g, ev):
    ks = {k["name"]: k for k in g["kernels"]}
    if "precompute_kernel" in ks:
        return SpecKernel(ks["precompute_kernel"]).store(ev, [])
    return ev


GOLDEN_SMALL = [("pwave", 1000), ("mass", 1000), ("spwave", 2000), ("cbpoly", 1000)]
# models without a C restatement: events from the GPU generator on the
# reference's one-stream partition (checked against the golden event hash)
REFERENCE_STREAM = ("spwave", "cbpoly")


@pytest.mark.parametrize("workload,n", GOLDEN_SMALL)
def test_fp64_matches_reference_golden(backend, workload, n):
    from morefit_gb300.workloads import Likelihood
    g = load_golden(f"{workload}_n{n}.json")
    ev = golden_events(workload, n)
    like = Likelihood(backend, g, np.float64)
    like.set_data(ev)
    cols = _cols(g, ev)
    for pt in g["points"]:
        for name in KERNELS:
            p = pt["kernel_params"][name]
            got = like.sums(name, param_vector=p)
            ref = np.array(pt["kernel_sums"][name])
            assert_sums_close(got, ref, _abs_scale(g, name, cols, p), what=f"{workload} {name}")


@pytest.mark.parametrize("workload,n", GOLDEN_SMALL)
def test_fitter_level_values(backend, workload, n):
    """likelihood / likelihood_and_gradient / hessian as the fitter returns them."""
    from morefit_gb300.workloads import Likelihood
    g = load_golden(f"{workload}_n{n}.json")
    like = Likelihood(backend, g, np.float64)
    like.set_data(golden_events(workload, n))
    for pt in g["points"]:
        nll = like.likelihood(pt["params"])
        assert abs(nll - pt["nll"]) <= 1e-10 * abs(pt["nll"])
        nll2, grad = like.likelihood_and_gradient(pt["params"])
        assert abs(nll2 - pt["nll_from_grad_kernel"]) <= 1e-10 * abs(pt["nll"])
        np.testing.assert_allclose(grad, pt["grad"], rtol=1e-8, atol=1e-9 * abs(pt["nll"]))
        h = like.hessian(pt["params"])
        np.testing.assert_allclose(h.ravel(), pt["hessian"], rtol=1e-8, atol=1e-9 * np.abs(pt["hessian"]).max())


@pytest.mark.parametrize("native", [True, False])
def test_precompute_matches_reference_text(backend, native):
    """Hoisted columns against the reference's precompute text. Native FP64
    within 1e-14; double-float (48-bit significands, inputs rounded to 48
    bits) within 3e-14 relative or 5e-15 absolute (the columns are of order
    0.1). Copied observables are bit-exact in both."""
    from morefit_gb300.workloads import Likelihood
    g = load_golden("pwave_n1000.json")
    ev = golden_events("pwave", 1000)
    like = Likelihood(backend, g, np.float64, native_f64=native)
    like.set_data(ev)
    got = like.pre.CopyFromOutputBuffer()
    ref = SpecKernel(kernel_spec(g, "precompute_kernel")).store(ev, [])
    assert np.array_equal(got[:3], ev)
    if native:
        np.testing.assert_allclose(got, ref, rtol=1e-14, atol=1e-15)
    else:
        np.testing.assert_allclose(got, ref, rtol=3e-14, atol=5e-15)


def test_double_float_functions(backend):
    """sqrt, sin, cos, log of double-float values (STORE kernel) against numpy
    FP64. Inputs are rounded to 48 bits first (relative error up to 2^-48), so
    the bars scale with the input where the function amplifies that: sin/cos
    within 6e-15 * (1 + |x|) absolute, sqrt within 1e-14 relative, log within
    2e-14 * (1 + |log y|) absolute (double-float additions round at about
    2^-47 of the result)."""
    from morefit_gb300.backend import CUDABlock
    rng = np.random.default_rng(11)
    n = 200000
    x = np.concatenate([rng.uniform(-4, 4, n // 4), rng.uniform(-60, 60, n // 4), rng.uniform(-7000, 7000, n // 4),
                        rng.normal(0, 1e-3, n // 4 - 6), [0.0, np.pi, -np.pi / 2, 5999.9, 6000.1, -1e-30]])
    # magnitudes from 1e-25 up: double-float keeps 48 bits down to about 2^-100
    y = np.concatenate([10.0 ** rng.uniform(-25, 30, n // 2), rng.uniform(0, 2, n // 2 - 3), [0.0, 1.0, 4.0]])
    blk = CUDABlock(backend, np.float64)
    blk.MakeComputeKernel("fn", n, ["x", "y"], ["s", "c", "q", "l"], [], ["sin(x)", "cos(x)", "sqrt(y)", "log(y)"],
                          False)
    blk.CopyToInputBuffer(np.stack([x, y]))
    blk.SetNevents(n)
    blk.SubmitKernel()
    s, c, q, lg = blk.CopyFromOutputBuffer()
    ax = 6e-15 * (1.0 + np.abs(x))
    assert np.all(np.abs(s - np.sin(x)) <= ax)
    assert np.all(np.abs(c - np.cos(x)) <= ax)
    np.testing.assert_allclose(q, np.sqrt(y), rtol=1e-14, atol=0)
    pos = y > 0
    err = np.abs(lg[pos] - np.log(y[pos])) / (1.0 + np.abs(np.log(y[pos])))
    w = int(np.argmax(err))
    assert err[w] <= 2e-14, (y[pos][w], lg[pos][w], np.log(y[pos][w]), err[w])
    assert lg[~pos][0] == -np.inf


@pytest.mark.parametrize("workload,n", [("pwave", 1000000), ("mass", 100000)])
def test_fp64_full_size_matches_reference(backend, oracle_lib, workload, n):
    from morefit_gb300.workloads import Likelihood
    g = load_golden(f"{workload}_n{n}.json")
    ev = oracle_lib.generate(workload, n)
    assert oracle_lib.fnv1a(ev) == g["events_fnv1a"]
    like = Likelihood(backend, g, np.float64)
    like.set_data(ev)
    cols = _cols(g, ev)
    for pt in g["points"]:
        for name in ("lh_kernel", "lh_grad_kernel"):
            p = pt["kernel_params"][name]
            got = like.sums(name, param_vector=p)
            ref = np.array(pt["kernel_sums"][name])
            assert_sums_close(got, ref, _abs_scale(g, name, cols, p), what=f"{workload} n={n} {name}")


@pytest.mark.parametrize("n", [1, 2, 3, 31, 32, 33, 255, 257, 511, 1000])
def test_edge_sizes(backend, n):
    from morefit_gb300.workloads import Likelihood
    g = load_golden("pwave_n1000.json")
    ev = golden_events("pwave", 1000)[:, :n]
    like = Likelihood(backend, g, np.float64)
    like.set_data(ev)
    cols = _cols(g, ev)
    for name in KERNELS:
        p = g["points"][2]["kernel_params"][name]
        ref = SpecKernel(kernel_spec(g, name)).reduce(cols, p)
        got = like.sums(name, param_vector=p)
        assert_sums_close(got, ref, _abs_scale(g, name, cols, p), what=f"n={n} {name}")


def test_deterministic(backend):
    from morefit_gb300.workloads import Likelihood
    g = load_golden("pwave_n1000.json")
    like = Likelihood(backend, g, np.float64)
    like.set_data(golden_events("pwave", 1000))
    p = g["points"][1]["kernel_params"]["lh_grad_kernel"]
    a = like.sums("lh_grad_kernel", param_vector=p)
    b = like.sums("lh_grad_kernel", param_vector=p)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("workload", ["pwave", "mass", "cbpoly"])
def test_combined_gradient_hessian_kernel(backend, workload):
    """The F + gradient + Hessian kernel (one launch, Hessian parameter buffers
    renamed) gives the two kernels' values: F and gradient within 1e-12 of
    the sum of absolute per-event terms, the Hessian within 1e-12 of its
    largest element. Models whose combined kernel would spill fall back to
    the two launches, with the same results."""
    from morefit_gb300.toystudy import SegmentLikelihood
    from morefit_gb300.workloads import Likelihood
    g = load_golden(f"{workload}_n1000.json")
    ev = golden_events(workload, 1000)
    like = Likelihood(backend, g, np.float64)
    like.set_data(ev)
    cols = _cols(g, ev)
    for pt in g["points"]:
        f, grad, h = like.value_gradient_hessian(pt["params"])
        f2, grad2 = like.likelihood_and_gradient(pt["params"])
        h2 = like.hessian(pt["params"])
        scale = 2.0 * _abs_scale(g, "lh_grad_kernel", cols, pt["kernel_params"]["lh_grad_kernel"])
        assert abs(f - f2) <= 1e-12 * scale[0]
        assert np.all(np.abs(grad - grad2) <= 1e-12 * scale[1:])
        assert np.all(np.abs(h - h2) <= 1e-12 * np.abs(h2).max())
    if workload == "pwave":
        assert like.combined_kernel() is not None
    # ragged segments through the same kernel: halves of the dataset
    sl = SegmentLikelihood(like, [0, 500], [500, 500])
    th = np.array([g["points"][0]["params"]] * 2)
    fs, gs, hs = sl.value_gradient_hessian(np.arange(2), th)
    f0, g0 = sl.value_and_gradient(np.arange(2), th)
    np.testing.assert_allclose(fs, f0, rtol=1e-12)
    np.testing.assert_allclose(gs, g0, rtol=1e-9, atol=1e-9 * np.abs(g0).max())
    np.testing.assert_allclose(hs, sl.hessian(np.arange(2), th), rtol=1e-9, atol=1e-12 * np.abs(hs).max())


@pytest.mark.parametrize("kernelT", [np.float64, np.float32])
def test_many_output_hessian_one_pass(backend, kernelT):
    """The S+P-wave Hessian (105 outputs). In double-float it is one kernel
    that neither spills nor reads the dataset more than once: the per-thread
    partials of the outputs beyond MF_NREG live in shared memory. In FP32 the
    single kernel spills and Likelihood splits its outputs into kernels of at
    most 36 that keep every partial in registers. Either way the sums equal,
    to 1e-12 (FP64) / 1e-6 (FP32) of the largest element, those of the other
    form (the FP64 split forced), single, batched and over ragged segments;
    the P-wave Hessian keeps all 36 partials in registers."""
    from morefit_gb300.toystudy import SegmentLikelihood, _unpack_hessian
    from morefit_gb300.workloads import Likelihood
    g = load_golden("spwave_n2000.json")
    ev = golden_events("spwave", 2000)
    like = Likelihood(backend, g, kernelT)
    like.set_data(ev)
    b = like.blocks["lh_hessian_kernel"]
    split = Likelihood(backend, g, kernelT)
    split.COMBINED_MAX_SPILL = -1  # the split into register-only parts, for FP64 forced
    split.set_data(ev)
    parts = split.kernel_parts("lh_hessian_kernel")
    assert len(parts) == 3
    assert all(split.blocks[p].kernel.info()["spill_bytes"] == 0 for p in parts)
    if kernelT == np.float64:
        assert like.kernel_parts("lh_hessian_kernel") == ["lh_hessian_kernel"]
        assert b.kernel.info()["spill_bytes"] == 0
        src = b.kernel.source()
        nreg = int(src.split("#define MF_NREG ")[1].split()[0])
        assert nreg < 105 and "mf_sacc[" in src
    else:
        assert len(like.kernel_parts("lh_hessian_kernel")) == 3
    tol = 1e-12 if kernelT == np.float64 else 1e-6
    for pt in g["points"]:
        pv = like.param_vector("lh_hessian_kernel", pt["params"])
        b.CopyToParameterBuffer(pv)
        b.SubmitKernel()
        whole = b.CopyFromKahanBuffer()  # the single kernel
        joined = split.sums("lh_hessian_kernel", pt["params"])
        assert joined.shape == whole.shape
        assert np.all(np.abs(joined - whole) <= tol * np.abs(whole).max())
        one = like.sums("lh_hessian_kernel", pt["params"])
        many = like.sums_many("lh_hessian_kernel", np.array([pt["params"]] * 2))
        assert np.array_equal(many[0], one) and np.array_equal(many[1], one)
    # ragged segments (the toy fits' Hessian): the golden events as one segment
    # and as three, against the single-dataset kernel
    counts = np.array([2000, 700, 1, 1299])
    begins = np.array([0, 0, 700, 701])
    th = np.array([pt["params"] for pt in g["points"]] + [g["points"][0]["params"]])
    npar = th.shape[1]
    for epb in (0, 512):
        sl = SegmentLikelihood(like, begins, counts, epb)
        hs = sl.hessian(np.arange(4), th)
        for s_ in range(4):
            b.CopyToParameterBuffer(like.param_vector("lh_hessian_kernel", th[s_]))
            if s_ == 0:
                b.SubmitKernel()
                whole = _unpack_hessian(b.CopyFromKahanBuffer()[None], npar)[0]
            else:
                one = b.SubmitSegments([begins[s_]], [counts[s_]], like.param_rows("lh_hessian_kernel", th[s_:s_ + 1]))
                whole = _unpack_hessian(one, npar)[0]
            assert np.all(np.abs(hs[s_] - whole) <= tol * np.abs(whole).max()), (epb, s_)
        # segments 1-3 at the same point cover the set once
        th3 = np.array([th[0]] * 3)
        parts3 = sl.hessian(np.arange(1, 4), th3).sum(0)
        assert np.all(np.abs(parts3 - hs[0]) <= tol * np.abs(hs[0]).max()), epb
    pw = Likelihood(backend, load_golden("pwave_n1000.json"), kernelT)
    assert pw.kernel_parts("lh_hessian_kernel") == ["lh_hessian_kernel"]
    psrc = pw.blocks["lh_hessian_kernel"].kernel.source()
    assert "#define MF_NREG 36" in psrc and "mf_sacc[" not in psrc


@pytest.mark.parametrize("workload", ["pwave", "mass", "mass_w"])
def test_sync_evaluation_equals_parameter_vector_path(backend, workload):
    """sums(kernel, theta), whose hoisted parameter buffers are evaluated in
    place in a preallocated vector, equals the evaluation from the explicit
    parameter vector bit for bit; that vector matches the fitter's own
    (fitter.hh:1059-1072) to rounding."""
    from morefit_gb300.workloads import Likelihood
    g = load_golden(f"{workload}_n1000.json")
    like = Likelihood(backend, g, np.float64)
    like.set_data(golden_events(workload, 1000))
    names = [k for k in KERNELS + ("lh_fisher_kernel",) if k in like.blocks]
    for pt in g["points"]:
        for name in names:
            pv = like.param_vector(name, pt["params"])
            np.testing.assert_allclose(pv, pt["kernel_params"][name], rtol=1e-13, atol=0)
            a = like.sums(name, pt["params"])
            assert np.array_equal(a, like.sums(name, param_vector=pv)), (workload, name)
            assert np.array_equal(a, like.sums(name, pt["params"]))


@pytest.mark.parametrize("workload,n", [("pwave", 1000), ("mass", 1000), ("pwave", 1000000), ("mass", 100000),
                                        ("spwave", 20000), ("cbpoly", 100000)])
def test_mixed_precision_parameter_shift(backend, oracle_lib, workload, n):
    """FP32 columns/arithmetic with FP64 sums move the estimate by at most 1e-3 sigma.

    The gradient error g32 - g64 shifts the minimum by dtheta = -H^-1 (g32 - g64)
    (H: FP64 Hessian of -2 ln L); sigma = sqrt(2 diag H^-1) (errordef 1 on
    -2 ln L, fitter.hh:72). Checked at every golden point; the NLL itself must
    agree to 1e-6 relative."""
    from morefit_gb300.workloads import Likelihood
    g = load_golden(f"{workload}_n{n}.json")
    if workload in REFERENCE_STREAM:
        ev = _reference_stream_events(backend, g, n)
    else:
        ev = golden_events(workload, n) if n == 1000 else oracle_lib.generate(workload, n)
    l64 = Likelihood(backend, g, np.float64)
    l64.set_data(ev)
    l32 = Likelihood(backend, g, np.float32)
    l32.set_data(ev)
    checked = []
    for ip, pt in enumerate(g["points"]):
        th = pt["params"]
        f64, g64 = l64.likelihood_and_gradient(th)
        f32, g32 = l32.likelihood_and_gradient(th)
        assert abs(f32 - f64) <= 1e-6 * abs(f64)
        h = l64.hessian(th)
        # the linearised shift needs a positive-definite Hessian (always at
        # the fitted minimum; the seven-parameter Crystal Ball model is not
        # convex half an error away from it)
        if np.linalg.eigvalsh(h).min() <= 0.0:
            continue
        hinv = np.linalg.inv(h)
        sigma = np.sqrt(2.0 * np.diag(hinv))
        shift = -hinv @ (g32 - g64) / sigma
        assert np.abs(shift).max() <= 1e-3, f"{workload} n={n}: shift/sigma {shift}"
        checked.append(ip)
    assert 1 in checked, checked


def _reference_stream_events(backend, g, n):
    """Events of the reference's generator run on one CPU thread: the GPU
    generator with a single xoshiro128++ stream (seed row 0) draws the same
    proposals in the same order; checked against the golden event hash."""
    from oracle import mforacle
    from morefit_gb300.workloads import generate_events
    ev = generate_events(backend, g, n, max_workitems=1).download()
    assert mforacle.fnv1a(ev) == g["events_fnv1a"], "GPU single-stream events differ from the reference's"
    return ev


@pytest.mark.parametrize("workload,n", [("cbpoly", 100000)])
def test_reference_stream_full_size_sums(backend, workload, n):
    """Crystal Ball + polynomial (conditionals, pow with a parameter
    exponent): NLL, gradient and Hessian sums over 100k events against the
    reference's at its three golden points."""
    from morefit_gb300.workloads import Likelihood
    g = load_golden(f"{workload}_n{n}.json")
    ev = _reference_stream_events(backend, g, n)
    like = Likelihood(backend, g, np.float64)
    like.set_data(ev)
    for pt in g["points"]:
        for name in KERNELS:
            p = pt["kernel_params"][name]
            got = like.sums(name, param_vector=p)
            ref = np.array(pt["kernel_sums"][name])
            assert_sums_close(got, ref, _abs_scale(g, name, ev, p), what=f"{workload} n={n} {name}")


def _per_value(backend, expr, cols, names):
    """One REDUCE output per value: a double-float REDUCE kernel over ragged
    segments of one event each."""
    from morefit_gb300.backend import CUDABlock
    blk = CUDABlock(backend, np.float64)
    blk.MakeComputeKernel("t", 0, names, ["r0"], [], [expr], True)
    blk.CopyToInputBuffer(cols)
    n = cols.shape[1]
    blk.SetNevents(n)
    out = blk.SubmitSegments(np.arange(n, dtype=np.uint64), np.ones(n, dtype=np.uint32), np.zeros((n, 0)))
    return out[:, 0], blk.kernel.fallback_count()


def test_double_float_exp_and_pow(backend):
    """exp and pow of double-float values in REDUCE kernels (table-driven
    exp on the FP32 pipe) against FP64: exp within 3e-14 relative over the
    FP32 normal range; pow within (|b ln a| + 1) * 3e-14; the IEEE special
    cases; results beyond the FP32 range come from the native-FP64 kernel.
    Below 2^-100 the low word of a double-float value is subnormal: those
    results are checked to an absolute 2^-147."""
    rng = np.random.default_rng(17)
    x = np.concatenate([rng.uniform(-87.0, 88.5, 20000), [0.0, -0.0, 1e-30, -1e-30, 1e-5, 0.5, 1.0, -1.0,
                                                          0.00541, -0.00541, 88.0, -87.0]]).astype(np.float32)
    got, fb = _per_value(backend, "exp(x)", x.astype(np.float64)[None, :], ["x"])
    ref = np.exp(x.astype(np.float64))
    # full precision while the low word is a normal float (results >= 2^-100);
    # below, a double-float value resolves about 2^-149
    full = ref >= 2.0 ** -100
    rel = np.abs(got - ref) / ref
    assert rel[full].max() < 3e-14, (rel[full].max(), x[full][np.argmax(rel[full])])
    assert np.all(np.abs(got - ref)[~full] <= 4 * 2.0 ** -149 + 3e-14 * ref[~full])
    assert fb == 0
    # an intermediate beyond the double-float range (the sums themselves are
    # combined in double-float and stay below 3.4e38): re-evaluated in FP64
    big = np.array([89.5, 95.0, 300.0], dtype=np.float64)
    got, fb = _per_value(backend, "(exp(x)*exp(-(x)))", big[None, :], ["x"])
    assert fb == 1 and np.allclose(got, 1.0, rtol=1e-15)
    tiny, _ = _per_value(backend, "exp(x)", np.array([[-110.0, -1e4]]), ["x"])
    assert np.all(tiny == 0.0)
    # pow: positive bases, real exponents
    a = rng.uniform(1e-3, 30.0, 20000).astype(np.float32).astype(np.float64)
    b = rng.uniform(-8.0, 8.0, 20000).astype(np.float32).astype(np.float64)
    got, _ = _per_value(backend, "pow(a,b)", np.vstack([a, b]), ["a", "b"])
    ref = np.power(a, b)
    rel = np.abs(got - ref) / ref
    bound = (np.abs(b * np.log(a)) + 1.0) * 3e-14
    assert np.all(rel <= bound), (rel / bound).max()
    # negative bases with integer exponents, zero, special exponents
    a = np.array([-2.0, -2.0, -3.5, -0.5, 0.0, 0.0, 0.0, 7.0, -7.0, -2.0, 1.0])
    b = np.array([3.0, 4.0, 2.0, -3.0, 2.5, -1.5, 0.0, 0.0, 0.0, 0.5, 123.25])
    got, _ = _per_value(backend, "pow(a,b)", np.vstack([a, b]), ["a", "b"])
    with np.errstate(invalid="ignore", divide="ignore"):
        ref = np.power(a, b)
    fin = np.isfinite(ref)
    np.testing.assert_allclose(got[fin], ref[fin], rtol=1e-13)
    # an infinite term leaves a compensated sum non-finite (inf or NaN: the
    # reference's Kahan step turns inf into NaN at the next term as well)
    assert not np.isfinite(got[~fin]).any()


def test_double_float_range_falls_back_to_native_fp64(backend):
    """At the 1000-event cbpoly minimum (alpha 0.95, n 8.5) the Hessian's tail
    terms reach pow(base, n)^4 ~ 1e52, beyond the FP32 exponent range of a
    double-float value: the reduction is evaluated again in native FP64 and
    agrees with the reference; the NLL kernel stays in double-float."""
    from morefit_gb300.workloads import Likelihood
    g = load_golden("cbpoly_n1000.json")
    ev = golden_events("cbpoly", 1000)
    like = Likelihood(backend, g, np.float64)
    like.set_data(ev)
    pt = g["points"][1]
    p = pt["kernel_params"]["lh_hessian_kernel"]
    got = like.sums("lh_hessian_kernel", param_vector=p)
    ref = np.array(pt["kernel_sums"]["lh_hessian_kernel"])
    assert_sums_close(got, ref, _abs_scale(g, "lh_hessian_kernel", ev, p), what="cbpoly hessian at the minimum")
    assert like.blocks["lh_hessian_kernel"].kernel.fallback_count() >= 1
    like.likelihood(pt["params"])
    assert like.blocks["lh_kernel"].kernel.fallback_count() == 0


def test_fit_matches_reference_cbpoly(backend):
    """Seven-parameter fit (Crystal Ball tail parameters included) of 100k
    events from the truth: values within 0.05 sigma and errors within 2e-3
    relative of the reference's MIGRAD + HESSE."""
    from morefit_gb300.workloads import Likelihood
    g = load_golden("cbpoly_n100000.json")
    like = Likelihood(backend, g, np.float64)
    like.set_data(_reference_stream_events(backend, g, 100000))
    limits = [(-0.2, 0.4), (0.01, 0.2), (0.5, 5.0), (1.5, 10.0), (-1.0, 1.0), (-1.0, 1.0), (0.0, 1.0)]
    r = like.fit(limits=limits)
    assert r.converged[0]
    ref_v = np.array(g["fit"]["values"])
    ref_e = np.array(g["fit"]["errors"])
    assert np.all(np.abs(r.values[0] - ref_v) <= 0.05 * ref_e), (r.values[0] - ref_v) / ref_e
    np.testing.assert_allclose(r.errors[0], ref_e, rtol=2e-3)


@pytest.mark.parametrize("n", [2000, 20000])
def test_gpu_generator_reproduces_reference_stream_spwave(backend, n):
    """The S+P-wave-with-acceptance density (no C restatement) through the
    GPU generator on the reference's one-stream partition gives the
    reference generator's events bit for bit."""
    g = load_golden(f"spwave_n{n}.json")
    ev = _reference_stream_events(backend, g, n)
    if n == 2000:
        assert np.array_equal(ev, golden_events("spwave", n))


@pytest.mark.parametrize("events_per_block", [0, 64, 256, 2048])
def test_ragged_segments(backend, events_per_block):
    """Segments of one event block at their own parameter rows, one block per
    segment (0) or in runs of ``events_per_block`` events combined per
    segment: each within the FP64 bar of the oracle, and a segment's sums the
    same bit for bit alone and among the others."""
    from morefit_gb300.workloads import Likelihood
    g = load_golden("pwave_n1000.json")
    ev = golden_events("pwave", 1000)
    like = Likelihood(backend, g, np.float64)
    like.set_data(ev)
    cols = _cols(g, ev)
    sk = SpecKernel(kernel_spec(g, "lh_grad_kernel"))
    counts = np.array([1, 0, 37, 200, 62, 300, 400], dtype=np.uint32)
    begins = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint64)
    rng = np.random.default_rng(7)
    rows = []
    for s in range(len(counts)):
        th = np.array(g["points"][s % 3]["params"]) + rng.normal(0, 0.01, 8)
        rows.append(like.param_vector("lh_grad_kernel", th))
    rows = np.array(rows)
    blk = like.blocks["lh_grad_kernel"]
    out = blk.SubmitSegments(begins, counts, rows, events_per_block)
    for s in range(len(counts)):
        sl = cols[:, begins[s]:begins[s] + counts[s]]
        ref = sk.reduce(sl, rows[s]) if counts[s] else np.zeros(9)
        scale = np.abs(sk.store(sl, rows[s])).sum(axis=1) if counts[s] else np.zeros(9)
        assert_sums_close(out[s], ref, scale, what=f"segment {s}")
        alone = blk.SubmitSegments(begins[s:s + 1], counts[s:s + 1], rows[s:s + 1], events_per_block)
        assert np.array_equal(alone[0], out[s]), f"segment {s} alone"


def test_prepared_columns_follow_writes(backend, oracle_lib):
    """REDUCE kernels read a prepared copy of their input (folded columns, FP64
    as float pairs). A write through the library, or a raw device write
    declared with mf_buffer_mark_modified, makes the next launch re-derive it."""
    import torch
    from morefit_gb300 import _lib as L
    from morefit_gb300.workloads import Likelihood
    g = load_golden("pwave_n1000.json")
    ev = golden_events("pwave", 1000)
    evb = np.ascontiguousarray(oracle_lib.generate("pwave", 2000, seed=12345)[:, 1000:])  # other events, same n
    p = g["points"][1]["kernel_params"]["lh_grad_kernel"]
    like = Likelihood(backend, g, np.float64)
    like.set_data(ev)
    a = like.sums("lh_grad_kernel", param_vector=p)
    like.set_data(evb)  # upload + precompute into the same buffers
    b = like.sums("lh_grad_kernel", param_vector=p)
    other = Likelihood(backend, g, np.float64)
    other.set_data(evb)
    assert np.array_equal(b, other.sums("lh_grad_kernel", param_vector=p))
    assert not np.allclose(a, b)
    # copy dataset A's hoisted columns into the buffer behind the library's back
    fresh = Likelihood(backend, g, np.float64)
    fresh.set_data(ev)
    dst, src = like.input_block("lh_grad_kernel").buf, fresh.input_block("lh_grad_kernel").buf
    nbytes = int(L.lib.mf_buffer_size(dst))
    assert nbytes == int(L.lib.mf_buffer_size(src))

    class _Dev:
        def __init__(self, ptr):
            self.__cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (ptr, False),
                                             "version": 3}

    backend.synchronize()
    torch.as_tensor(_Dev(L.lib.mf_buffer_device_ptr(dst)), device="cuda").copy_(
        torch.as_tensor(_Dev(L.lib.mf_buffer_device_ptr(src)), device="cuda"))
    torch.cuda.synchronize()
    L.check(L.lib.mf_buffer_mark_modified(dst))
    assert np.array_equal(like.sums("lh_grad_kernel", param_vector=p), a)


@pytest.mark.parametrize("mixed_n", [False, True])
def test_batched_evaluations_match_single(backend, oracle_lib, mixed_n):
    """mf_kernel_reduce_many (evaluations overlapping their predecessors' tails)
    gives bit-identical sums to one mf_kernel_reduce per evaluation, also when
    one buffer appears with two event counts in a batch."""
    import ctypes as C
    from morefit_gb300 import _lib as L
    from morefit_gb300.workloads import Likelihood
    g = load_golden("pwave_n1000.json")
    n = 20000
    sets = []
    for seed in range(3):
        like = Likelihood(backend, g, np.float64)
        like.set_data(oracle_lib.generate("pwave", n, seed=1000 + seed))
        sets.append(like)
    k = sets[0].blocks["lh_grad_kernel"].kernel
    order = [0, 1, 2, 0, 2, 1, 1, 0] * 4
    counts = [n - 5003 * (i % 2) if (mixed_n and o == 0) else n for i, o in enumerate(order)]
    rows = np.array([g["points"][i % 3]["kernel_params"]["lh_grad_kernel"] for i in range(len(order))])
    single = np.zeros((len(order), k.nout))
    for i, o in enumerate(order):
        blk = sets[o].input_block()
        L.check(L.lib.mf_kernel_reduce(k.handle, blk.buf, blk.stride, counts[i], L.dptr(rows[i]), rows.shape[1],
                                       L.dptr(single[i])))
    ins = (L.c_buf * len(order))(*[sets[o].input_block().buf for o in order])
    strides = np.array([sets[o].input_block().stride for o in order], np.uint64)
    ns = np.array(counts, np.uint64)
    out = L.c_buf()
    L.check(L.lib.mf_buffer_alloc(backend.handle, single.nbytes, C.byref(out)))
    u64p = C.POINTER(C.c_uint64)
    L.check(L.lib.mf_kernel_reduce_many(k.handle, len(order), ins, strides.ctypes.data_as(u64p),
                                        ns.ctypes.data_as(u64p), L.dptr(np.ascontiguousarray(rows)), rows.shape[1],
                                        out))
    got = np.zeros_like(single)
    L.check(L.lib.mf_buffer_d2h(out, 0, got.ctypes.data, got.nbytes))
    L.check(L.lib.mf_buffer_free(out))
    assert np.isfinite(single).all()
    assert np.array_equal(got, single)


def test_budget_covers_prepared_copies():
    """The prepared copy of an input is allocated against the context's HBM budget."""
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import CUDABackend
    from morefit_gb300.workloads import Likelihood
    g = load_golden("pwave_n1000.json")
    n = 100000
    ev = np.tile(golden_events("pwave", 1000), (1, n // 1000))
    # raw (3 columns) + hoisted (14 columns) FP64 fit in the budget; the 9 prepared columns do not
    need = 17 * 8 * n
    b = CUDABackend(0, hbm_budget_bytes=need + (1 << 20))
    like = Likelihood(b, g, np.float64)
    like.set_data(ev)
    with pytest.raises(L.MFError, match="BUDGET"):
        like.sums("lh_grad_kernel", param_vector=g["points"][1]["kernel_params"]["lh_grad_kernel"])
    del like
    b.close()


def test_budget_is_enforced():
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import CUDABackend, DeviceColumns
    b = CUDABackend(0, hbm_budget_bytes=1 << 20)
    cols = DeviceColumns(b, L.MF_F64)
    cols.ensure(1, 1000)
    with pytest.raises(L.MFError, match="BUDGET"):
        DeviceColumns(b, L.MF_F64).ensure(3, 1 << 20)
    cols.free()
    b.close()


@pytest.mark.parametrize("workload,n", [("pwave", 1000), ("pwave", 20000), ("mass", 30000)])
def test_gpu_generator_matches_oracle(backend, oracle_lib, workload, n):
    """GPU accept-reject with the accelerator partition equals the C restatement event by event."""
    from morefit_gb300.workloads import generate_events, generate_partition, load_spec
    spec = load_spec(workload)
    cols = generate_events(backend, spec, n)
    got = cols.download()
    nper, nseeds = generate_partition(n)
    ref = oracle_lib.generate_partitioned(workload, n, nper, nseeds)
    same = np.all(got == ref, axis=0)
    assert same.mean() > 0.999, f"only {same.mean():.4f} of events identical"
    # any difference is a rare accept flip at the threshold; then the stream shifts within one thread only
    assert np.allclose(np.sort(got[0]), np.sort(ref[0]), atol=0.05) or same.all()


@pytest.mark.parametrize("elem,n,ncols", [(0, 1, 1), (0, 1000, 3), (0, 1000003, 5), (1, 777777, 4)])
def test_columns_sum(backend, elem, n, ncols):
    """Device column sums equal exact sums (math.fsum) to double-float accuracy."""
    import ctypes as C
    import math
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import DeviceColumns
    rng = np.random.default_rng(n + ncols)
    host = rng.normal(0.3, 2.0, size=(ncols, n))
    if elem == L.MF_F32:
        host = host.astype(np.float32)
    cols = DeviceColumns(backend, elem)
    cols.upload(host)
    sums = np.zeros(ncols)
    L.check(L.lib.mf_columns_sum(cols.buf, elem, ncols, n, cols.stride, L.dptr(sums)))
    for c in range(ncols):
        exact = math.fsum(host[c].astype(np.float64))
        scale = np.abs(host[c].astype(np.float64)).sum()
        assert abs(sums[c] - exact) <= 1e-13 * scale, (c, sums[c], exact)
    again = np.zeros(ncols)
    L.check(L.lib.mf_columns_sum(cols.buf, elem, ncols, n, cols.stride, L.dptr(again)))
    assert np.array_equal(sums, again)
