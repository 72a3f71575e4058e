"""Host linear algebra of the batched fits (mf_spd_solve_batch) against
LAPACK through numpy: Newton steps -H^-1 g and diag(H^-1) per matrix, for
orders on the lane-interleaved path (p <= 16) and the one-matrix path, batch
sizes that are not multiples of the lane count, and matrices that are not
positive definite (reported, then solved by LAPACK). CPU only."""
import numpy as np
import pytest


@pytest.mark.parametrize("n,p", [(1, 1), (5, 3), (13, 8), (4096, 8), (9, 16), (7, 20), (3, 64)])
def test_spd_solve_batch_matches_lapack(n, p):
    from morefit_gb300.toystudy import _inverse_diagonal, _newton_steps, _spd_solve
    rng = np.random.default_rng(n * 100 + p)
    a = rng.normal(size=(n, p, p))
    h = a @ a.transpose(0, 2, 1) + 0.5 * np.eye(p)
    g = rng.normal(size=(n, p))
    nonpd = [t for t in (2, 11) if t < n]
    for t in nonpd:
        h[t] = -h[t]
    x, dinv, ok = _spd_solve(h, g)
    assert list(np.nonzero(~ok)[0]) == nonpd
    ref = np.linalg.solve(h, g[..., None])[..., 0]
    good = ok
    scale = np.abs(ref).max(axis=1, keepdims=True)
    assert np.all(np.abs(x[good] - ref[good]) <= 1e-12 * scale[good])
    dref = np.einsum("tii->ti", np.linalg.inv(h))
    assert np.all(np.abs(dinv[good] - dref[good]) <= 1e-12 * np.abs(dref[good]))
    # the fitter's entry points fall back to LAPACK for the rest
    np.testing.assert_allclose(_newton_steps(h, g), -ref, rtol=1e-12, atol=1e-12 * scale.max())
    np.testing.assert_allclose(_inverse_diagonal(h), dref, rtol=1e-12)


def test_spd_solve_batch_rejects_bad_orders():
    import ctypes as C
    from morefit_gb300 import _lib as L
    h = np.eye(3)[None]
    ok = np.zeros(1, np.uint8)
    with pytest.raises(L.MFError):
        L.check(L.lib.mf_spd_solve_batch(1, 0, L.dptr(h), None, None, None, ok.ctypes.data_as(C.POINTER(C.c_uint8))))
    with pytest.raises(L.MFError):
        L.check(L.lib.mf_spd_solve_batch(1, 65, L.dptr(h), None, None, None, ok.ctypes.data_as(C.POINTER(C.c_uint8))))
