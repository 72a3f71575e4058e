"""Host side of the serving benchmark (no GPU): the request stream's mix,
sizes and arrivals, and the latency summary."""
import math

import numpy as np


def test_request_stream_mix_sizes_and_arrivals():
    from morefit_gb300.serving import poisson_stream
    n, rate = 20000, 300.0
    reqs = poisson_stream(n, rate, seed=3)
    assert [r.id for r in reqs] == list(range(n))
    # 60% mass fits, 40% S+P-wave fits
    frac = sum(r.model == "mass" for r in reqs) / n
    assert abs(frac - 0.6) < 0.02
    assert {r.model for r in reqs} == {"mass", "spwave"}
    # event counts log-uniform in [1k, 5M]
    sizes = np.array([r.nevents for r in reqs])
    assert sizes.min() >= 1000 and sizes.max() <= 5_000_000
    logs = np.log(sizes)
    lo, hi = math.log(1000), math.log(5_000_000)
    assert abs(logs.mean() - 0.5 * (lo + hi)) < 0.05
    assert abs(logs.std() - (hi - lo) / math.sqrt(12)) < 0.05
    # Poisson arrivals: increasing, exponential gaps of mean 1/rate
    t = np.array([r.arrival for r in reqs])
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert np.all(gaps > 0)
    assert abs(gaps.mean() * rate - 1.0) < 0.03
    assert abs(gaps.std() / gaps.mean() - 1.0) < 0.05
    # every request its own dataset seed
    assert len({r.seed for r in reqs}) == n


def test_request_stream_is_reproducible():
    from morefit_gb300.serving import poisson_stream
    a = poisson_stream(50, 100.0, seed=7)
    b = poisson_stream(50, 100.0, seed=7)
    c = poisson_stream(50, 100.0, seed=8)
    key = lambda rs: [(r.model, r.nevents, r.seed, r.arrival) for r in rs]
    assert key(a) == key(b)
    assert key(a) != key(c)


def test_latency_summary():
    from morefit_gb300.serving import FitOutcome, ServerStats, latency_summary
    st = ServerStats(ticks=5, batched_calls=7, evaluations=40, max_active=3, peak_bytes=2_500_000_000)
    lat = np.linspace(0.001, 0.100, 100)
    for i, l in enumerate(lat):
        st.outcomes.append(FitOutcome(i, "mass", 1000, np.zeros(4), np.ones(4), 0.0, 6, i != 50,
                                      admitted=0.0, finished=0.5 + 0.01 * i, latency=float(l)))
    s = latency_summary(st)
    assert s["fits"] == 100
    assert math.isclose(s["fits_per_s"], 100 / (0.5 + 0.99))
    assert math.isclose(s["p50_ms"], float(np.percentile(lat, 50)) * 1e3)
    assert math.isclose(s["p99_ms"], float(np.percentile(lat, 99)) * 1e3)
    assert s["max_active"] == 3 and s["batched_calls"] == 7 and s["evaluations"] == 40
    assert math.isclose(s["peak_resident_GB"], 2.5)
    assert s["all_converged"] is False
