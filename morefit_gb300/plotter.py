"""Projections of a fitted model on the data: the reference's plotter
(include/plotter.hh).

``plotter::plot`` (plotter.hh:220-470) integrates the normalised density over
npdf_bins = nbins * pdf_bin_multiplier bins of one variable (the other
dimensions over their full ranges) with an "integral_kernel" built from
PDF::definite_integral() (plotter.hh:138-216), histograms the data (weighted
when the data carry an event weight), scales the PDF to the histogram, forms
residuals and pulls, and writes a matplotlib script (.py) or a ROOT macro
(.C).

Here the integral is a STORE kernel on the GPU in native FP64 (one row per
bin; the reference substitutes the parameter values into the kernel text,
this kernel takes them at launch, with the parameter-only terms hoisted into
buffers as the fitter does), the histogram is ``mf_histogram`` over the
device-resident event column, and the host arithmetic and the output text
restate plotter.hh:285-470 line by line (C++ stream formatting: ``%g``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _lib as L
from .backend import CUDABackend, CUDABlock, DeviceColumns, ExpressionSet


@dataclass
class PlotterOptions:
    """plotter_options (plotter.hh:44-70); float fields are C++ floats."""
    plotter: str = "root"             # "root" (.C macro) or "matplotlib" (.py script)
    pdf_bin_multiplier: int = 10
    plot_width: int = 1200
    aspect_ratio: float = 4.0 / 3.0
    plot_pulls: bool = False
    pull_fraction: float = 0.20
    max_pull: float = 3.0
    print_level: int = 2


@dataclass
class PlotResult:
    variable: str
    range: tuple
    pdf_y: np.ndarray      # (npdf_bins,) integral of the density over each fine bin
    y: np.ndarray          # (nbins,) events (or sum of weights) per bin
    dy: np.ndarray         # (nbins,) sqrt(y) (or sqrt(sum of w^2))
    pulls: np.ndarray      # (nbins,)
    pdf_scale: float
    text: str              # the written file


def _g(v) -> str:
    """A double as `ostream << v` prints it (default precision 6)."""
    return "%g" % float(v)


def _f32(v) -> float:
    return float(np.float32(v))


def _seq_sum(a) -> float:
    t = 0.0
    for v in np.asarray(a, dtype=np.float64).tolist():
        t += v
    return t


def _join(vals, end: str) -> str:
    return ", ".join(_g(v) for v in vals) + end


class Plotter:
    """plotter<...> (plotter.hh:96-135) on the CUDA backend."""

    def __init__(self, options: PlotterOptions, backend: CUDABackend):
        self.opts = options
        self.backend = backend
        self._blocks = {}
        self._hist = None

    def _integral_block(self, spec: dict, variable: str) -> tuple:
        key = (spec["workload"], variable)
        if key not in self._blocks:
            integ = spec["integrals"][variable]
            blk = CUDABlock(self.backend, np.float64, native_f64=True)
            blk.MakeComputeKernel("integral_kernel", 0, integ["inputs"], ["integral"], integ["params"],
                                  integ["exprs"], False)
            exprs = ExpressionSet(spec["parameters"], [e for _, e in integ["buffers"]]) if integ["buffers"] else None
            self._blocks[key] = (blk, exprs)
        return self._blocks[key]

    def integrals(self, spec: dict, theta, variable: str, edges_from: np.ndarray, edges_to: np.ndarray) -> np.ndarray:
        """Integral of the normalised density over [from_i, to_i) of `variable`."""
        blk, exprs = self._integral_block(spec, variable)
        th = np.asarray(theta, dtype=np.float64)[None, :]
        pv = th[0] if exprs is None else np.concatenate([th, exprs.eval(th)], axis=1)[0]
        blk.CopyToInputBuffer(np.vstack([edges_from, edges_to]))
        blk.SetNevents(len(edges_from))
        blk.CopyToParameterBuffer(pv)
        blk.SubmitKernel()
        return blk.CopyFromOutputBuffer()[0].astype(np.float64)

    def histogram(self, data: DeviceColumns, col: int, weight_col, lo: float, hi: float, nbins: int):
        """(y, sum of w^2, events outside [lo, hi)) of one device column."""
        if self._hist is None or self._hist[1] < nbins:
            b = L.c_buf()
            L.check(L.lib.mf_buffer_alloc(self.backend.handle, (2 * nbins + 1) * 8, C.byref(b)))
            if self._hist is not None:
                L.check(L.lib.mf_buffer_free(self._hist[0]))
            self._hist = (b, nbins)
        hb = self._hist[0]
        base = L.lib.mf_buffer_device_ptr(hb)
        item = data.itemsize
        dptr = L.lib.mf_buffer_device_ptr(data.buf)
        x = dptr + col * data.stride * item
        w = None if weight_col is None else dptr + weight_col * data.stride * item
        stream = C.c_void_p()
        L.check(L.lib.mf_context_stream(self.backend.handle, C.byref(stream)))
        L.check(L.lib.mf_histogram(x, w, data.elem, data.n, float(lo), float(hi), nbins, base, base + nbins * 8,
                                   base + 2 * nbins * 8, stream))
        out = np.empty(2 * nbins + 1, dtype=np.float64)
        self.backend.synchronize()
        L.check(L.lib.mf_buffer_d2h(hb, 0, out.ctypes.data, out.nbytes))
        return out[:nbins].copy(), out[nbins:2 * nbins].copy(), int(out[2 * nbins:].view(np.uint64)[0])

    def plot(self, spec: dict, theta, data, variable: str, filename: str, nbins: int = 100, range_min: float = 0.0,
             range_max: float = 0.0) -> PlotResult:
        """plotter::plot (plotter.hh:220-470): writes `filename` (.py for
        matplotlib, .C for ROOT) and returns the numbers it holds. `data` is
        a device event block with the spec's dimensions as columns, or a host
        array (ndims, n) that is uploaded."""
        dims = list(spec["dimensions"])
        if variable not in dims:
            raise ValueError(f"Variable {variable} not found, unable to plot.")
        if not isinstance(data, DeviceColumns):
            cols = DeviceColumns(self.backend, L.MF_F64)
            cols.upload(np.asarray(data, dtype=np.float64))
            data = cols
        varidx = dims.index(variable)
        if range_min == range_max:
            range_min, range_max = spec["ranges"][varidx]
        mult = self.opts.pdf_bin_multiplier
        npdf_bins = nbins * mult
        dx = (range_max - range_min) / float(npdf_bins)
        i = np.arange(npdf_bins, dtype=np.float64)
        pdf_y = self.integrals(spec, theta, variable, range_min + i * dx, range_min + (i + 1.0) * dx)

        weight = spec.get("weight")
        wcol = dims.index(weight) if weight else None
        y, y2, outside = self.histogram(data, varidx, wcol, range_min, range_max, nbins)
        if outside:
            raise ValueError(f"{outside} events outside [{range_min}, {range_max}) of {variable}")
        tex = spec.get("tex", dims)[varidx]
        res = finish_plot(self.opts, filename, variable, tex, range_min, range_max, nbins, pdf_y, y, y2)
        Path(filename).write_text(res.text)
        return res


def finish_plot(opts: PlotterOptions, filename: str, variable: str, tex: str, lo: float, hi: float, nbins: int,
                pdf_y, y, y2) -> PlotResult:
    """The host part of plotter::plot after the integrals and the histogram
    (plotter.hh:285-470): y2 is the sum of squared weights per bin (y itself
    without weights); returns the numbers and the file text."""
    mult = opts.pdf_bin_multiplier
    npdf_bins = nbins * mult
    pdf_y = np.asarray(pdf_y, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    dy = np.sqrt(np.asarray(y2, dtype=np.float64))
    hist_int = _seq_sum(y)
    pdf_int = _seq_sum(pdf_y)
    pdf_scale = hist_int / pdf_int * npdf_bins / float(nbins)
    residuals = np.zeros(nbins)
    for k in range(npdf_bins):
        ib = k // mult
        residuals[ib] += (y[ib] - pdf_y[k] * pdf_scale) / mult
    pulls = residuals / dy
    if opts.max_pull > 0.0:
        max_pull = _f32(opts.max_pull)
    else:
        max_pull = 0.0
        for p in pulls:
            if abs(p) > max_pull:
                max_pull = abs(p)
        max_pull *= 1.05
    writer = _matplotlib if opts.plotter == "matplotlib" else _root
    text = writer(opts, filename, tex, lo, hi, nbins, npdf_bins, y, dy, pulls, pdf_y, hist_int, pdf_int, max_pull)
    return PlotResult(variable, (lo, hi), pdf_y, y, dy, pulls, pdf_scale, text)


# ---- output text (plotter.hh:365-470) ----
def _matplotlib(o, filename, tex, lo, hi, nbins, npdf_bins, y, dy, pulls, pdf_y, hist_int, pdf_int, max_pull):
    if Path(filename).suffix != ".py":
        raise ValueError(f"Unknown file extension: {filename}")
    stem = Path(filename).stem
    t = "import matplotlib.pyplot as plt\nimport numpy as np\nplt.rcParams['text.usetex'] = True\n"
    t += (f"x = np.linspace({_g(lo + 0.5 * (hi - lo) / float(nbins))}, "
          f"{_g(hi - 0.5 * (hi - lo) / float(nbins))}, {nbins})\n")
    t += f"dx = [{_g(0.5 * (hi - lo) / float(nbins))} for x in range({nbins})]\n"
    t += "y = [" + _join(y, "]\n")
    t += "dy = [" + _join(0.5 * dy, "]\n")
    if o.plot_pulls:
        t += "y_pull = [" + _join(pulls, "]\n")
    hist_max = y[0]
    for v in y:
        if v > hist_max:
            hist_max = v
    t += (f"x_pdf = np.linspace({_g(lo + 0.5 * (hi - lo) / float(npdf_bins))}, "
          f"{_g(hi - 0.5 * (hi - lo) / float(npdf_bins))}, {npdf_bins})\n")
    t += "y_pdf = [" + _join([p * hist_int / pdf_int * npdf_bins / float(nbins) for p in pdf_y], "]\n")
    label = tex.replace("#", "\\")
    if o.plot_pulls:
        pf = _f32(o.pull_fraction)
        t += (f"fig, ax = plt.subplots(nrows=2, ncols=1,  layout='constrained', height_ratios=[{_g(1.0 - pf)}, "
              f"{_g(pf)}])\n")
        t += "ax[0].plot(x_pdf, y_pdf, linestyle='solid', color='red')\n"
        t += "ax[0].errorbar(x, y, xerr=dx, yerr=dy, linestyle='none', marker='o', markersize=2, color='black')\n"
        t += f"ax[0].set_xlabel('${label}$')\n"
        t += "ax[0].set_ylabel('$\\mathrm{events}$')\n"
        t += f"ax[0].set_xlim({_g(lo)}, {_g(hi)})\n"
        t += f"ax[0].set_ylim({_g(0.0)}, {_g(hist_max * 1.15)})\n"
        t += (f"ax[1].bar(x=x, height=y_pull, width={_g((hi - lo) / float(nbins))}, facecolor='gray', "
              "linestyle='solid', edgecolor='black')\n")
        t += f"#ax[1].set_xlabel('${label}$')\n"
        t += "ax[1].set_ylabel('$\\mathrm{pull}$')\n"
        t += f"ax[1].set_xlim({_g(lo)}, {_g(hi)})\n"
        t += f"ax[1].set_ylim(-{_g(max_pull)}, {_g(max_pull)})\n"
    else:
        t += "fig, ax = plt.subplots()\n"
        t += "ax.plot(x_pdf, y_pdf, linestyle='solid', color='red')\n"
        t += "ax.errorbar(x, y, xerr=dx, yerr=dy, linestyle='none', marker='o', markersize=2, color='black')\n"
        t += f"ax.set_xlabel('${label}$')\n"
        t += "ax.set_ylabel('$\\mathrm{events}$')\n"
        t += f"plt.xlim({_g(lo)}, {_g(hi)})\n"
        t += f"plt.ylim({_g(0.0)}, {_g(hist_max * 1.15)})\n"
    t += "plt.show()\n"
    t += f"fig.savefig(\"{stem}.pdf\", bbox_inches='tight')\n"
    return t

def _root(o, filename, tex, lo, hi, nbins, npdf_bins, y, dy, pulls, pdf_y, hist_int, pdf_int, max_pull):
    if Path(filename).suffix != ".C":
        raise ValueError(f"Unknown file extension: {filename}")
    stem = Path(filename).stem
    pf = _f32(o.pull_fraction)
    t = f"int {stem}() {{\n"
    t += ("gROOT->SetStyle(\"Plain\");\ngStyle->SetOptFit(0);\ngStyle->SetOptStat(0);\n"
          "gStyle->SetTextFont(132);\ngStyle->SetTextSize(0.06);\ngStyle->SetTitleFont(132,\"xyz\");\n"
          "gStyle->SetLabelFont(132,\"xyz\");\ngStyle->SetLabelSize(0.05,\"xyz\");\n"
          "gStyle->SetTitleSize(0.06,\"xyz\");\n")
    t += (f"TCanvas* c0 = new TCanvas(\"c0\", \"c0\", {o.plot_width}, "
          f"{_g(o.plot_width / _f32(o.aspect_ratio))});\n")
    t += f"TH1D* hist = new TH1D(\"hist\", \";{tex};events\", {nbins}, {_g(lo)}, {_g(hi)});\n"
    t += f"double hist_values[{len(y)}] = {{" + _join(y, "};\n")
    t += f"double hist_errors[{len(dy)}] = {{" + _join(dy, "};\n")
    t += (f"for (unsigned int i=0; i<{len(y)}; i++)\n{{\n  hist->SetBinContent(i+1, hist_values[i]);\n"
          "  hist->SetBinError(i+1, hist_errors[i]);\n}\n")
    t += f"TH1D* hist_pdf = new TH1D(\"hist_pdf\", \";{tex};events\", {npdf_bins}, {_g(lo)}, {_g(hi)});\n"
    t += f"double pdf_values[{len(pdf_y)}] = {{" + _join(pdf_y, "};\n")
    t += f"double pdf_errors[{len(pdf_y)}] = {{" + _join(np.zeros(len(pdf_y)), "};\n")
    t += (f"for (unsigned int i=0; i<{len(pdf_y)}; i++)\n{{\n  hist_pdf->SetBinContent(i+1, pdf_values[i]);\n"
          "  hist_pdf->SetBinError(i+1, pdf_errors[i]);\n}\n")
    t += f"hist_pdf->Scale(hist->Integral()/hist_pdf->Integral()*{npdf_bins}/double({nbins}));\n"
    if o.plot_pulls:
        t += f"TH1D* pull_hist = new TH1D(\"pull_hist\", \";{tex};pull\", {nbins}, {_g(lo)}, {_g(hi)});\n"
        t += f"double pull_values[{len(pulls)}] = {{" + _join(pulls, "};\n")
        t += (f"for (unsigned int i=0; i<{len(pulls)}; i++)\n{{\n"
              "  pull_hist->SetBinContent(i+1, pull_values[i]);\n  pull_hist->SetBinError(i+1, 0.0);\n}\n"
              "c0->cd(0);\n"
              f"TPad *hist_pad = new TPad(\"hist_pad\",\"\",0.0, {_g(pf)}, 1.0, 1.0);\n"
              "hist_pad->SetMargin(0.125,0.05,0.125,0.05);\nhist_pad->Draw();\nhist_pad->cd();\n"
              "hist->SetMinimum(0.0);\nhist->Draw(\"e\");\nhist_pdf->SetLineColor(2);\n"
              "hist_pdf->SetLineWidth(2.0);\nhist_pdf->Draw(\"lcsame\");\nc0->cd(0);\n"
              f"TPad *pull_pad = new TPad(\"pull_pad\",\"\",0.0, 0.0, 1.0, {_g(pf)});\n"
              "pull_pad->SetMargin(0.125,0.05,0.125,0.125);\npull_pad->Draw();\npull_pad->cd();\n"
              "pull_hist->SetFillColor(kGray);\n"
              f"pull_hist->GetYaxis()->SetTitleOffset(1.0*{_g(pf / (1.0 - pf))});\n"
              f"pull_hist->GetYaxis()->SetLabelSize(0.05*{_g((1.0 - pf) / pf)});\n"
              f"pull_hist->GetYaxis()->SetTitleSize(0.06*{_g((1.0 - pf) / pf)});\n"
              "pull_hist->GetXaxis()->SetLabelSize(0);\npull_hist->GetXaxis()->SetTitleSize(0);\n"
              f"pull_hist->SetMinimum(-{_g(max_pull)});\npull_hist->SetMaximum(+{_g(max_pull)});\n"
              "pull_hist->Draw(\"hist\");\n"
              "TGaxis *axis = new TGaxis(pull_hist->GetXaxis()->GetXmin(), pull_hist->GetMaximum(), "
              "pull_hist->GetXaxis()->GetXmax(), pull_hist->GetMaximum(), pull_hist->GetXaxis()->GetXmin(), "
              "pull_hist->GetXaxis()->GetXmax(), 510, \"-U\");\n"
              "axis->Draw();\n"
              f"c0->Print(\"{stem}.eps\", \"eps\");\n"
              "delete hist;\ndelete hist_pdf;\ndelete hist_pad;\ndelete pull_hist;\ndelete pull_pad;\n"
              "delete c0;\n")
    else:
        t += ("c0->cd()->SetMargin(0.125,0.05,0.125,0.05);\nhist->SetMinimum(0.0);\nhist->Draw(\"e\");\n"
              "hist_pdf->SetLineColor(2);\nhist_pdf->SetLineWidth(2.0);\nhist_pdf->Draw(\"lcsame\");\n"
              f"c0->Print(\"{stem}.eps\", \"eps\");\n"
              "delete hist;\ndelete hist_pdf;\ndelete c0;\n")
    t += "return 1;\n}\n"
    return t
