"""The reference's plotter (include/plotter.hh): per-bin integrals of the
density, the data histogram, pulls and the written matplotlib / ROOT text.

Golden files (oracle/refkit plot) hold the reference's own output: the
integral kernel's per-bin values at full precision and the .py and .C files
it wrote for 100k generated events at the truth. CPU tests feed the
reference's integrals and a restated histogram through finish_plot and
require the same file text byte for byte; GPU tests run the whole plot
(integral kernel in native FP64, mf_histogram) and require integrals within
1e-12 relative and the same text.
"""
import numpy as np
import pytest

from conftest import load_golden

PLOTS = [("mass", "m"), ("mass_w", "m"), ("pwave", "ctl"), ("pwave", "ctk"), ("pwave", "phi"), ("cbpoly", "x")]
CPU_PLOTS = [p for p in PLOTS if p[0] != "cbpoly"]  # cbpoly events come from the GPU generator


def _events(oracle_lib, g):
    ev = oracle_lib.generate(g["workload"], g["nevents"])
    assert oracle_lib.fnv1a(ev) == g["events_fnv1a"]
    return ev


def _histogram(x, w, lo, hi, nbins):
    """plotter.hh:296-319: bin floor((x - lo)/(hi - lo)*nbins), sequential sums."""
    idx = np.floor((x - lo) / (hi - lo) * nbins).astype(np.int64)
    assert idx.min() >= 0 and idx.max() < nbins
    y = np.zeros(nbins)
    y2 = np.zeros(nbins)
    if w is None:
        np.add.at(y, idx, 1.0)
        return y, y.copy()
    np.add.at(y, idx, w)
    np.add.at(y2, idx, w * w)
    return y, y2


@pytest.mark.parametrize("workload,var", CPU_PLOTS)
def test_plot_text_reproduces_reference(oracle_lib, tmp_path, workload, var):
    from morefit_gb300.plotter import PlotterOptions, finish_plot
    from morefit_gb300.workloads import load_spec
    g = load_golden(f"plot_{workload}_{var}.json")
    spec = load_spec(workload)
    ev = _events(oracle_lib, g)
    dims = spec["dimensions"]
    lo, hi = g["range"]
    w = ev[dims.index(spec["weight"])] if spec.get("weight") else None
    y, y2 = _histogram(ev[dims.index(var)], w, lo, hi, g["nbins"])
    for kind, ext in (("matplotlib", "py"), ("root", "C")):
        opts = PlotterOptions(plotter=kind, plot_pulls=True)
        name = str(tmp_path / f"plot_{workload}_{var}.{ext}")
        res = finish_plot(opts, name, var, g["tex"][dims.index(var)], lo, hi, g["nbins"], g["pdf_y"], y, y2)
        assert res.text == g[ext], f"{ext} text differs"


def test_plot_options_without_pulls(tmp_path):
    """The no-pull layouts (plotter.hh:418-429, :512-523) and a file extension
    the chosen plotter does not write."""
    from morefit_gb300.plotter import PlotterOptions, finish_plot
    pdf = np.full(20, 0.05)
    y = np.arange(1.0, 3.0)
    res = finish_plot(PlotterOptions(plotter="matplotlib"), str(tmp_path / "a.py"), "m", "m", 0.0, 1.0, 2, pdf, y, y)
    assert "fig, ax = plt.subplots()\n" in res.text and "y_pull" not in res.text
    res = finish_plot(PlotterOptions(), str(tmp_path / "a.C"), "m", "m", 0.0, 1.0, 2, pdf, y, y)
    assert "pull_hist" not in res.text and res.text.endswith("return 1;\n}\n")
    with pytest.raises(ValueError):
        finish_plot(PlotterOptions(), str(tmp_path / "a.py"), "m", "m", 0.0, 1.0, 2, pdf, y, y)


@pytest.mark.gpu
@pytest.mark.parametrize("workload,var", PLOTS)
def test_gpu_plot_matches_reference(oracle_lib, tmp_path, workload, var):
    from morefit_gb300.backend import CUDABackend
    from morefit_gb300.plotter import Plotter, PlotterOptions
    from morefit_gb300.workloads import generate_events, load_spec
    g = load_golden(f"plot_{workload}_{var}.json")
    spec = load_spec(workload)
    b = CUDABackend(0)
    try:
        if workload == "cbpoly":  # the reference's one-stream partition on the GPU generator
            ev = generate_events(b, spec, g["nevents"], max_workitems=1).download()
            assert oracle_lib.fnv1a(ev) == g["events_fnv1a"]
        else:
            ev = _events(oracle_lib, g)
        for kind, ext in (("matplotlib", "py"), ("root", "C")):
            pl = Plotter(PlotterOptions(plotter=kind, plot_pulls=True), b)
            res = pl.plot(spec, g["truth"], ev, var, str(tmp_path / f"plot_{workload}_{var}.{ext}"), g["nbins"])
            np.testing.assert_allclose(res.pdf_y, g["pdf_y"], rtol=1e-12, atol=1e-15)
            dims = spec["dimensions"]
            w = ev[dims.index(spec["weight"])] if spec.get("weight") else None
            y, y2 = _histogram(ev[dims.index(var)], w, g["range"][0], g["range"][1], g["nbins"])
            if w is None:
                assert np.array_equal(res.y, y)
            else:
                np.testing.assert_allclose(res.y, y, rtol=1e-12)
                np.testing.assert_allclose(res.dy ** 2, y2, rtol=1e-12)
            assert res.text == g[ext], f"{ext} text differs"
    finally:
        b.close()


@pytest.mark.gpu
def test_gpu_histogram_edges_and_outside(tmp_path):
    """Events at hi, below lo and NaN are reported outside (the reference
    throws for them); float columns bin like double ones."""
    import ctypes as C
    from morefit_gb300 import _lib as L
    from morefit_gb300.backend import CUDABackend, DeviceColumns
    from morefit_gb300.plotter import Plotter, PlotterOptions
    b = CUDABackend(0)
    try:
        pl = Plotter(PlotterOptions(), b)
        x = np.array([0.0, 0.25, 0.5, 0.999999, 1.0, -0.1, np.nan, 0.75])
        for elem, dt in ((L.MF_F64, np.float64), (L.MF_F32, np.float32)):
            cols = DeviceColumns(b, elem)
            cols.upload(x[None, :].astype(dt))
            y, y2, outside = pl.histogram(cols, 0, None, 0.0, 1.0, 4)
            assert outside == 3
            assert np.array_equal(y, [1.0, 1.0, 1.0, 2.0]) and np.array_equal(y2, y)
        # more bins than the shared-memory histogram holds
        rng = np.random.default_rng(1)
        x = rng.uniform(0.0, 1.0, 200000)
        w = rng.uniform(0.5, 1.5, 200000)
        cols = DeviceColumns(b, L.MF_F64)
        cols.upload(np.vstack([x, w]))
        for nbins in (3000, 10000):
            y, y2, outside = pl.histogram(cols, 0, None, 0.0, 1.0, nbins)
            ref, _ = _histogram(x, None, 0.0, 1.0, nbins)
            assert outside == 0 and np.array_equal(y, ref)
            y, y2, outside = pl.histogram(cols, 0, 1, 0.0, 1.0, nbins)
            ry, ry2 = _histogram(x, w, 0.0, 1.0, nbins)
            np.testing.assert_allclose(y, ry, rtol=1e-12)
            np.testing.assert_allclose(y2, ry2, rtol=1e-12)
    finally:
        b.close()
