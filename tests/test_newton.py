"""The serving loop's Newton coroutine on the host (no GPU): driven by an
analytic objective, the combined form (F, gradient and Hessian from one
request, at the start and at every step trial) reaches the same minimum,
errors and convergence as the form with separate gradient and Hessian
requests, in no more requests."""
import numpy as np
import pytest


def _objective(x):
    """F(x) = sum a_i (x_i - c_i)^2 + b (x_0 x_1)^2: smooth, minimum at c
    with c_0 = 0 (so the quartic term vanishes there)."""
    a = np.array([2.0, 0.5, 3.0])
    c = np.array([0.0, 0.3, -0.2])
    b = 0.7
    d = x - c
    f = float(np.sum(a * d * d) + b * (x[0] * x[1]) ** 2)
    g = 2.0 * a * d
    g[0] += 2.0 * b * x[0] * x[1] ** 2
    g[1] += 2.0 * b * x[1] * x[0] ** 2
    h = np.diag(2.0 * a)
    h[0, 0] += 2.0 * b * x[1] ** 2
    h[1, 1] += 2.0 * b * x[0] ** 2
    h[0, 1] = h[1, 0] = 4.0 * b * x[0] * x[1]
    return f, g, h


def _drive(co):
    req = co.send(None)
    n = 0
    try:
        while True:
            kind, x = req
            f, g, h = _objective(np.asarray(x))
            n += 1
            req = co.send({"grad": (f, g), "hess": h, "gh": (f, g, h)}[kind])
    except StopIteration as stop:
        return stop.value, n


@pytest.mark.parametrize("start", [[0.8, -0.5, 0.4], [-1.5, 1.2, 0.9]])
def test_combined_requests_reach_the_same_minimum(start):
    from morefit_gb300.serving import newton_fit
    limits = [(-5.0, 5.0)] * 3
    (x1, e1, f1, c1, _), n1 = _drive(newton_fit(start, limits, edm_tol=1e-12))
    (x2, e2, f2, c2, _), n2 = _drive(newton_fit(start, limits, edm_tol=1e-12, combined=True))
    assert c1 and c2
    np.testing.assert_allclose(x2, x1, atol=1e-7)
    np.testing.assert_allclose(x2, [0.0, 0.3, -0.2], atol=1e-6)
    np.testing.assert_allclose(e2, e1, rtol=1e-5)
    assert abs(f2 - f1) <= 1e-12
    assert n2 <= n1
