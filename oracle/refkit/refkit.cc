// Oracle kit driver: runs the reference's unchanged generator, fitter and
// Minuit2 on seeded synthetic events and writes golden vectors as JSON.
//
// TEST INFRASTRUCTURE ONLY (built by oracle/Makefile into oracle/_ref/ from
// the reference sources where they lie; never shipped, never on the product
// path). Workloads:
//   mass  : fsig*Gauss(m; mb, sigma) + (1-fsig)*Exp(alpha*m) on m in
//           [5000,5600] (pdf.hh:139-194, :423-484, :486-651), 4 floating
//           parameters, fitter options of benchmarking/morefit_massfit.cc:77-99
//           but with analytic gradient and Hessian.
//   pwave : KstarmumuAngularPDF (physicspdfs.hh:28-214) on ctl, ctk in
//           [-1,1], phi in [-pi,pi], 8 floating parameters, fitter options of
//           benchmarking/morefit_kstarmumu.cc:74-92.
//   spwave: the P-wave density plus S-wave and S-P interference terms times
//           a Legendre acceptance (SPwaveAccPDF below), 14 floating parameters.
//   mass_w: the mass model with an event weight column (weighted fit with
//           the Fisher kernel and the covariance correction).
//   cbpoly: Crystal Ball + quadratic polynomial on x in [-1,1] (pdf.hh:199-419,
//           :717-892), 7 floating parameters.
// Events come from generator::generate on the accelerator path with one
// xoshiro128++ stream seeded by Xoshiro128pp::setSeed(229387429)
// (random.hh:355-362, generator.hh:102-113), as in the reference drivers.
//
// Usage:
//   refkit golden <workload> <nevents> <out.json> [events.bin]
//   refkit bench  <mass|pwave|spwave> <nevents> <nthreads> <nevals>
//   refkit toys   <pwave> <ntoys> <mean events> <jitter> <out.json> [seed]
//   refkit plot   <workload> <nevents> <variable> <nbins> <out.py> <out.json>
//   refkit fitfile <workload> <datasets.bin> <out.json>
//   refkit fitevents <workload> <events.f64> <nthreads>
//   refkit benchevents <workload> <events.f64> <nthreads> <nevals> <max seconds>
#define MOREFIT_H 1  // keep graph.hh from pulling in the OpenCL/LLVM backends
#include <cassert>
#include <chrono>
#include <cmath>
#include <fstream>
#include <functional>
#include <cstdint>
#include <cstdio>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "graph.hh"
#include "eventvector.hh"
#include "parametervector.hh"
#include "pdf.hh"
#include "physicspdfs.hh"
#include "compute.hh"
#include "gcc_block.hh"
#include "fitter.hh"
#include "Math/MinimizerOptions.h"
#include "generator.hh"
#include "plotter.hh"
#include "random.hh"

using namespace morefit;
typedef double kT;
typedef double eT;
typedef LLVMBackend backendT;
typedef LLVMBlock<kT, eT> blockT;

// ---- capture hooks: every parameter vector and Kahan result, per kernel ----
struct Capture {
  std::map<std::string, std::vector<double>> params, sums, outputs;
};
static Capture* g_capture = nullptr;
static void install_capture() {
  block_observer() = [](const std::string& kernel, const char* what, const std::vector<double>& v) {
    if (!g_capture) return;
    const std::string w = what;
    if (w == "params")
      g_capture->params[kernel] = v;
    else if (w == "sums")
      g_capture->sums[kernel] = v;
    else
      g_capture->outputs[kernel] = v;
  };
}

static std::string jstr(const std::string& s) {
  std::string o = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') {
      o += '\\';
      o += c;
    } else if (c == '\n') {
      o += "\\n";
    } else if (static_cast<unsigned char>(c) < 0x20) {
      char b[8];
      std::snprintf(b, sizeof b, "\\u%04x", unsigned(c));
      o += b;
    } else {
      o += c;
    }
  }
  return o + "\"";
}
static std::string jnum(double v) {
  if (std::isnan(v)) return "null";
  char b[64];
  std::snprintf(b, sizeof b, "%.17g", v);
  return b;
}
static std::string jvec(const std::vector<double>& v) {
  std::string o = "[";
  for (size_t i = 0; i < v.size(); i++) o += (i ? "," : "") + jnum(v[i]);
  return o + "]";
}
static std::string jsvec(const std::vector<std::string>& v) {
  std::string o = "[";
  for (size_t i = 0; i < v.size(); i++) o += (i ? "," : "") + jstr(v[i]);
  return o + "]";
}

static uint64_t fnv1a(const void* p, size_t n) {
  const unsigned char* b = (const unsigned char*)p;
  uint64_t h = 1469598103934665603ULL;
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 1099511628211ULL;
  }
  return h;
}
#include "workloads.hh"

typedef Workload<kT, eT> WorkloadT;
static WorkloadT make_workload(const std::string& which) { return make_workload<kT, eT>(which); }


static void generate(WorkloadT& w, backendT* backend, Xoshiro128pp* rnd, unsigned n, EventVector<kT, eT>& out) {
  generator_options gen_opts;
  gen_opts.rndtype = generator_options::randomization_type::on_accelerator;
  gen_opts.print_level = 0;
  generator<kT, eT, backendT, blockT> gen(&gen_opts, backend, rnd);
  gen.generate(n, w.pdf, w.params, out);
  if (w.weight) {
    // Weights w_i = 0.5 + frac(i * 0.6180339887498949) in [0.5, 1.5), a
    // deterministic sequence uncorrelated with the generated events.
    out.add_dimensions({w.weight});
    const unsigned d = out.ndimensions() - 1;
    for (unsigned i = 0; i < n; i++) {
      double f = double(i) * 0.6180339887498949;
      f -= std::floor(f);
      out(i, d) = 0.5 + f;
    }
    out.set_event_weight(w.weight->get_name());
  }
}

// Parses "<prefix><name> = <expr>" lines printed by fitter::make_kernels at print_level 2.
static std::vector<std::pair<std::string, std::string>> grab(const std::string& log, const std::string& prefix) {
  std::vector<std::pair<std::string, std::string>> r;
  std::istringstream is(log);
  std::string line;
  while (std::getline(is, line)) {
    if (line.rfind(prefix, 0) != 0) continue;
    std::string rest = line.substr(prefix.size());
    size_t eq = rest.find(" = ");
    if (eq == std::string::npos) continue;
    r.push_back({rest.substr(0, eq), rest.substr(eq + 3)});
  }
  return r;
}
static std::string jpairs(const std::vector<std::pair<std::string, std::string>>& v) {
  std::string o = "[";
  for (size_t i = 0; i < v.size(); i++) o += (i ? "," : "") + ("[" + jstr(v[i].first) + "," + jstr(v[i].second) + "]");
  return o + "]";
}

static int cmd_golden(const std::string& which, unsigned n, const std::string& out_json, const std::string& out_bin) {
  compute_options copts;
  copts.llvm_nthreads = 1;
  copts.print_kernel = false;
  backendT backend(&copts);
  WorkloadT w = make_workload(which);
  Xoshiro128pp rnd;
  rnd.setSeed(int64_t(229387429));
  EventVector<kT, eT> data(w.dims);
  recorded_kernels().clear();
  generate(w, &backend, &rnd, n, data);
  std::vector<RecordedKernel> gen_records = recorded_kernels();
  const uint64_t ev_hash = fnv1a(data.get_data(), data.buffer_size());
  if (!out_bin.empty()) {
    FILE* f = std::fopen(out_bin.c_str(), "wb");
    std::fwrite(data.get_data(), 1, data.buffer_size(), f);
    std::fclose(f);
  }
  std::vector<double> truth;
  for (auto* p : w.params) truth.push_back(p->get_value());

  fitter_options fopts = make_fit_opts(w);
  fopts.print_level = 2;  // make_kernels prints the hoisted buffer expressions
  fitter<kT, eT, backendT, blockT> fit(&fopts, &backend);
  recorded_kernels().clear();
  // fit() runs make_kernels once (a second make_kernels on one fitter would
  // re-grow its result dimension vectors, fitter.hh:544).
  std::ostringstream captured;
  auto* old = std::cout.rdbuf(captured.rdbuf());
  auto t0 = std::chrono::steady_clock::now();
  fit.fit(w.pdf, w.params, &data);
  auto t1 = std::chrono::steady_clock::now();
  std::cout.rdbuf(old);
  fopts.print_level = 0;
  std::string log = captured.str();
  std::vector<double> values, errors;
  for (auto* p : w.params) {
    values.push_back(p->get_value());
    errors.push_back(p->get_error());
  }
  const int npar = int(w.params.size());

  // Evaluation points: truth, fitted minimum, and a displaced point.
  std::vector<std::vector<double>> points = {truth, values};
  {
    std::vector<double> d = truth;
    // half an error from the truth, alternating in sign, kept within each
    // parameter's limits (a poorly constrained parameter would leave them)
    for (int i = 0; i < npar; i++)
      d[i] = std::min(std::max(truth[i] + 0.5 * errors[i] * ((i % 2) ? -1.0 : 1.0), w.params[i]->get_min()),
                      w.params[i]->get_max());
    points.push_back(d);
  }
  std::string pts = "[";
  for (size_t k = 0; k < points.size(); k++) {
    for (int i = 0; i < npar; i++) w.params[i]->set_value(points[k][i]);
    Capture cap;
    g_capture = &cap;
    std::cout.rdbuf(captured.rdbuf());
    double nll = fit.likelihood();
    std::vector<double> grad(npar);
    double nll2 = fit.likelihood_and_gradient(npar, grad.data());
    std::vector<double> h(npar * npar);
    fit.hessian(npar, h.data());
    std::vector<double> fm;
    if (w.weight) {
      fm.resize(size_t(npar) * npar);
      fit.fisher(w.pdf, w.params, &data, npar, fm.data());
    }
    std::cout.rdbuf(old);
    g_capture = nullptr;
    pts += std::string(k ? "," : "") + "{\"params\":" + jvec(points[k]) + ",\"nll\":" + jnum(nll) +
           ",\"nll_from_grad_kernel\":" + jnum(nll2) + ",\"grad\":" + jvec(grad) + ",\"hessian\":" + jvec(h) +
           (w.weight ? ",\"fisher\":" + jvec(fm) : std::string()) + ",\"kernel_params\":{";
    bool first = true;
    for (auto& kv : cap.params) {
      pts += std::string(first ? "" : ",") + jstr(kv.first) + ":" + jvec(kv.second);
      first = false;
    }
    pts += "},\"kernel_sums\":{";
    first = true;
    for (auto& kv : cap.sums) {
      pts += std::string(first ? "" : ",") + jstr(kv.first) + ":" + jvec(kv.second);
      first = false;
    }
    pts += "}}";
  }
  pts += "]";

  std::string kern = "[";
  std::vector<RecordedKernel> all = gen_records;
  for (auto& r : recorded_kernels()) all.push_back(r);
  for (size_t i = 0; i < all.size(); i++) {
    auto& r = all[i];
    kern += std::string(i ? "," : "") + "{\"name\":" + jstr(r.name) + ",\"inputs\":" + jsvec(r.inputs) +
            ",\"outputs\":" + jsvec(r.outputs) + ",\"params\":" + jsvec(r.params) + ",\"exprs\":" + jsvec(r.exprs) +
            ",\"kahan\":" + (r.kahan ? "true" : "false");
    if (r.generate)
      kern += ",\"generate\":true,\"lo\":" + jvec(r.lo) + ",\"hi\":" + jvec(r.hi) + ",\"maxprob\":" + jnum(r.maxprob);
    kern += "}";
  }
  kern += "]";
  std::vector<std::string> dnames, pnames;
  for (auto* d : w.dims) dnames.push_back(d->get_name());
  if (w.weight) dnames.push_back(w.weight->get_name());
  for (auto* p : w.params) pnames.push_back(p->get_name());
  char hash[32];
  std::snprintf(hash, sizeof hash, "%016llx", (unsigned long long)ev_hash);
  std::string js = "{\"workload\":" + jstr(w.name) + ",\"nevents\":" + std::to_string(n) +
                   ",\"seed\":229387429,\"events_fnv1a\":" + jstr(hash) + ",\"dimensions\":" + jsvec(dnames) +
                   ",\"parameters\":" + jsvec(pnames) + ",\"truth\":" + jvec(truth) +
                   ",\"maxprob\":" + jnum(w.pdf->get_max()) + ",\"kernels\":" + kern +
                   ",\"event_buffers\":" + jpairs(grab(log, "EVENTBUFFER ")) +
                   ",\"lh_buffers\":" + jpairs(grab(log, "BUFFER ")) +
                   ",\"grad_buffers\":" + jpairs(grab(log, "GRADBUFFER: ")) +
                   ",\"hessian_buffers\":" + jpairs(grab(log, "HESSIANBUFFER: ")) +
                   (w.weight ? ",\"weight\":" + jstr(w.weight->get_name()) +
                                   ",\"fisher_buffers\":" + jpairs(grab(log, "FISHERBUFFER: "))
                             : std::string()) +
                   ",\"fit\":{\"values\":" +
                   jvec(values) + ",\"errors\":" + jvec(errors) + ",\"wall_ms\":" +
                   jnum(std::chrono::duration<double, std::milli>(t1 - t0).count()) + "},\"points\":" + pts + "}\n";
  FILE* f = std::fopen(out_json.c_str(), "w");
  std::fputs(js.c_str(), f);
  std::fclose(f);
  std::fprintf(stderr, "golden %s n=%u events_fnv1a=%s fit_ms=%.1f\n", which.c_str(), n, hash,
               std::chrono::duration<double, std::milli>(t1 - t0).count());
  return 0;
}

// Times NLL+gradient evaluations of the reference kernel text at nthreads.
static int cmd_bench(const std::string& which, unsigned n, unsigned nthreads, unsigned nevals) {
  compute_options copts;
  copts.llvm_nthreads = 1;
  copts.print_kernel = false;
  backendT backend(&copts);
  WorkloadT w = make_workload(which);
  Xoshiro128pp rnd;
  rnd.setSeed(int64_t(229387429));
  EventVector<kT, eT> data(w.dims);
  generate(w, &backend, &rnd, n, data);
  copts.llvm_nthreads = nthreads;
  fitter_options fopts = make_fit_opts(w);
  fopts.minuit_maxcalls = 1;
  fopts.minuit_maxiterations = 1;
  fopts.postrun_hesse = false;
  fitter<kT, eT, backendT, blockT> fit(&fopts, &backend);
  std::ostringstream sink;
  auto* old = std::cout.rdbuf(sink.rdbuf());
  fit.fit(w.pdf, w.params, &data);
  const int npar = int(w.params.size());
  std::vector<double> grad(npar);
  for (int i = 0; i < 3; i++) fit.likelihood_and_gradient(npar, grad.data());
  auto t0 = std::chrono::steady_clock::now();
  double acc = 0;
  for (unsigned i = 0; i < nevals; i++) acc += fit.likelihood_and_gradient(npar, grad.data());
  auto t1 = std::chrono::steady_clock::now();
  std::cout.rdbuf(old);
  double s = std::chrono::duration<double>(t1 - t0).count();
  std::printf("{\"workload\":\"%s\",\"nevents\":%u,\"nthreads\":%u,\"nevals\":%u,\"evals_per_s\":%.6g,\"nll\":%.17g}\n",
              which.c_str(), n, nthreads, nevals, nevals / s, acc / nevals);
  return 0;
}

// Toy study with the reference's own generator and fitter, one toy at a
// time as toystudy::toy does (toystudy.hh:55-82), except that every toy's
// truth is the workload's truth times (1 + u), u uniform in [-jitter, jitter]
// (SplitMix64 stream), and the event count is the reference's
// RandomGenerator::poisson(mean) (random.hh:42-80) clipped to [200, 50000].
// Each toy is generated at its truth (the generate kernel is rebuilt per toy
// because the generator substitutes the parameter values into it,
// generator.hh:145) and fitted from it (MIGRAD + HESSE). Writes the pulls.
static int cmd_toys(const std::string& which, unsigned ntoys, double mean, double jitter, const std::string& out,
                    uint64_t seed = 229387429) {
  compute_options copts;
  copts.llvm_nthreads = 1;
  copts.print_kernel = false;
  backendT backend(&copts);
  WorkloadT w = make_workload(which);
  Xoshiro128pp rnd;
  rnd.setSeed(int64_t(seed));
  generator_options gen_opts;
  gen_opts.rndtype = generator_options::randomization_type::on_accelerator;
  gen_opts.print_level = 0;
  generator<kT, eT, backendT, blockT> gen(&gen_opts, &backend, &rnd);
  fitter_options fopts = make_fit_opts(w);
  fitter<kT, eT, backendT, blockT> fit(&fopts, &backend);
  std::vector<double> base;
  for (auto* p : w.params) base.push_back(p->get_value());
  uint64_t sm = 0x746f79737475ULL + (seed - 229387429);
  auto uni = [&sm]() {
    sm += 0x9e3779b97f4a7c15ULL;
    uint64_t z = sm;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return double((z ^ (z >> 31)) >> 11) * 0x1.0p-53;
  };
  std::string pulls = "[", truths = "[", counts = "[";
  unsigned nconv = 0;
  std::ostringstream sink;
  auto* old = std::cout.rdbuf(sink.rdbuf());
  for (unsigned t = 0; t < ntoys; t++) {
    std::vector<double> truth(base.size());
    for (size_t i = 0; i < base.size(); i++) truth[i] = base[i] * (1.0 + jitter * (2.0 * uni() - 1.0));
    for (size_t i = 0; i < base.size(); i++) {
      w.params[i]->set_value(truth[i]);
      w.params[i]->set_start_value(truth[i]);
    }
    unsigned n = rnd.poisson(mean);
    n = std::min(50000u, std::max(200u, n));
    EventVector<kT, eT> data(w.dims, n);
    gen.generate(n, w.pdf, w.params, data, false);
    for (size_t i = 0; i < base.size(); i++) w.params[i]->set_value(truth[i]);
    const bool ok = fit.fit(w.pdf, w.params, &data, t > 0);
    nconv += ok ? 1 : 0;
    std::vector<double> pl;
    for (size_t i = 0; i < base.size(); i++)
      pl.push_back((w.params[i]->get_value() - truth[i]) / w.params[i]->get_error());
    pulls += std::string(t ? "," : "") + jvec(pl);
    truths += std::string(t ? "," : "") + jvec(truth);
    counts += std::string(t ? "," : "") + std::to_string(n);
  }
  std::cout.rdbuf(old);
  std::string js = "{\"workload\":" + jstr(which) + ",\"ntoys\":" + std::to_string(ntoys) + ",\"mean\":" + jnum(mean) +
                   ",\"jitter\":" + jnum(jitter) + ",\"converged\":" + std::to_string(nconv) + ",\"counts\":" +
                   counts + "],\"truths\":" + truths + "],\"pulls\":" + pulls + "]}\n";
  FILE* f = std::fopen(out.c_str(), "w");
  std::fputs(js.c_str(), f);
  std::fclose(f);
  std::fprintf(stderr, "toys %s: %u of %u fits converged\n", which.c_str(), nconv, ntoys);
  return 0;
}

// Runs the reference's plotter (matplotlib output, pulls on) on generated
// events at the truth and records: the integral kernel it builds (parameter
// values substituted, plotter.hh:138-216) with its per-bin integrals, the
// written .py text, and the same definite integral with the parameters kept
// as names (parameter-only terms hoisted into buffers as the fitter does),
// for a backend that takes parameter values at launch.
static int cmd_plot(const std::string& which, unsigned n, const std::string& var, unsigned nbins,
                    const std::string& out_py, const std::string& out_json) {
  compute_options copts;
  copts.llvm_nthreads = 1;
  copts.print_kernel = false;
  backendT backend(&copts);
  WorkloadT w = make_workload(which);
  Xoshiro128pp rnd;
  rnd.setSeed(int64_t(229387429));
  EventVector<kT, eT> data(w.dims);
  generate(w, &backend, &rnd, n, data);
  const uint64_t ev_hash = fnv1a(data.get_data(), data.buffer_size());

  plotter_options popts;
  popts.plotter = plotter_options::plotter_type::MatPlotLib;
  popts.plot_pulls = true;
  popts.print_level = 0;
  plotter<kT, eT, backendT, blockT> pl(&popts, &backend);
  recorded_kernels().clear();
  Capture cap;
  g_capture = &cap;
  std::ostringstream captured;
  auto* old = std::cout.rdbuf(captured.rdbuf());
  pl.plot(w.pdf, w.params, &data, var, out_py, "", nbins);
  // the same plot as a ROOT macro (same stem, kernels reused)
  const std::string out_c = out_py.substr(0, out_py.size() - 3) + ".C";
  popts.plotter = plotter_options::plotter_type::Root;
  pl.plot(w.pdf, w.params, &data, var, out_c, "", nbins, 0.0, 0.0, true);
  std::cout.rdbuf(old);
  g_capture = nullptr;
  RecordedKernel rk;
  for (auto& r : recorded_kernels())
    if (r.name == "integral_kernel") rk = r;
  std::vector<double> pdf_y = cap.outputs["integral_kernel"];
  pdf_y.resize(size_t(nbins) * popts.pdf_bin_multiplier);

  // the integral with symbolic parameters (plotter::make_kernels without the
  // parameter substitution)
  std::vector<std::string> dn, floating;
  std::vector<eT> dv;
  std::string vfrom, vto;
  double lo = 0.0, hi = 0.0;
  for (auto* d : w.pdf->dimensions())
    if (d->get_name() != var) {
      dn.push_back(d->get_from_name());
      dv.push_back(d->get_min());
      dn.push_back(d->get_to_name());
      dv.push_back(d->get_max());
    } else {
      vfrom = d->get_from_name();
      vto = d->get_to_name();
      lo = d->get_min();
      hi = d->get_max();
    }
  for (auto* p : w.params) floating.push_back(p->get_name());
  std::unique_ptr<ComputeGraphNode<kT, eT>> integral = w.pdf->definite_integral()->substitute(dn, dv)->simplify();
  integral->rename_variable(vfrom, "morefit_from");
  integral->rename_variable(vto, "morefit_to");
  std::vector<std::string> bnames;
  std::vector<std::unique_ptr<ComputeGraphNode<kT, eT>>> bexprs;
  std::unique_ptr<ComputeGraphNode<kT, eT>> sym =
      integral->optimize_buffering_constant_terms(bnames, bexprs, floating, "morefit_parambuffer_", 2.0);
  std::vector<std::pair<std::string, std::string>> bufs;
  for (size_t i = 0; i < bnames.size(); i++) bufs.push_back({bnames[i], bexprs[i]->get_kernel()});
  std::vector<std::string> sparams = floating;
  for (auto& b : bnames) sparams.push_back(b);

  std::ifstream pyf(out_py), cf(out_c);
  std::stringstream pys, cs;
  pys << pyf.rdbuf();
  cs << cf.rdbuf();
  std::vector<std::string> tex;
  for (auto* d : w.pdf->dimensions()) tex.push_back(d->get_tex());
  std::vector<double> truth;
  for (auto* p : w.params) truth.push_back(p->get_value());
  char hash[32];
  std::snprintf(hash, sizeof hash, "%016llx", (unsigned long long)ev_hash);
  std::string js = "{\"workload\":" + jstr(w.name) + ",\"nevents\":" + std::to_string(n) +
                   ",\"events_fnv1a\":" + jstr(hash) + ",\"variable\":" + jstr(var) +
                   ",\"nbins\":" + std::to_string(nbins) +
                   ",\"pdf_bin_multiplier\":" + std::to_string(popts.pdf_bin_multiplier) +
                   ",\"range\":" + jvec({lo, hi}) + ",\"parameters\":" + jsvec(floating) +
                   ",\"truth\":" + jvec(truth) + ",\"reference_kernel\":{\"inputs\":" + jsvec(rk.inputs) +
                   ",\"params\":" + jsvec(rk.params) + ",\"exprs\":" + jsvec(rk.exprs) +
                   "},\"pdf_y\":" + jvec(pdf_y) + ",\"integral\":{\"inputs\":" +
                   jsvec({"morefit_from", "morefit_to"}) + ",\"params\":" + jsvec(sparams) +
                   ",\"exprs\":" + jsvec({sym->get_kernel()}) + ",\"buffers\":" + jpairs(bufs) +
                   "},\"tex\":" + jsvec(tex) + ",\"py\":" + jstr(pys.str()) + ",\"C\":" + jstr(cs.str()) +
                   "}\n";
  FILE* f = std::fopen(out_json.c_str(), "w");
  std::fputs(js.c_str(), f);
  std::fclose(f);
  std::fprintf(stderr, "plot %s %s n=%u bins=%u events_fnv1a=%s\n", which.c_str(), var.c_str(), n, nbins, hash);
  return 0;
}

// Fits datasets from a file with the reference's fitter: the file holds, per
// dataset, uint32 n, npar doubles (truth, also the start point) and the SoA
// events (ndims x n doubles). Writes values and errors per dataset.
static int cmd_fitfile(const std::string& which, const std::string& in, const std::string& out) {
  compute_options copts;
  copts.llvm_nthreads = 1;
  copts.print_kernel = false;
  backendT backend(&copts);
  WorkloadT w = make_workload(which);
  fitter_options fopts = make_fit_opts(w);
  fitter<kT, eT, backendT, blockT> fit(&fopts, &backend);
  FILE* f = std::fopen(in.c_str(), "rb");
  if (!f) return 2;
  const size_t npar = w.params.size(), nd = w.dims.size();
  std::string vals = "[", errs = "[";
  std::ostringstream sink;
  auto* old = std::cout.rdbuf(sink.rdbuf());
  for (unsigned t = 0;; t++) {
    uint32_t n = 0;
    if (std::fread(&n, 4, 1, f) != 1) break;
    std::vector<double> truth(npar);
    if (std::fread(truth.data(), 8, npar, f) != npar) break;
    EventVector<kT, eT> data(w.dims, n);
    if (std::fread(data.get_data(), 8, nd * n, f) != nd * n) break;
    for (size_t i = 0; i < npar; i++) {
      w.params[i]->set_value(truth[i]);
      w.params[i]->set_start_value(truth[i]);
    }
    fit.fit(w.pdf, w.params, &data, t > 0);
    std::vector<double> v, e;
    for (auto* p : w.params) {
      v.push_back(p->get_value());
      e.push_back(p->get_error());
    }
    vals += std::string(t ? "," : "") + jvec(v);
    errs += std::string(t ? "," : "") + jvec(e);
  }
  std::cout.rdbuf(old);
  std::fclose(f);
  FILE* o = std::fopen(out.c_str(), "w");
  std::fputs(("{\"values\":" + vals + "],\"errors\":" + errs + "]}\n").c_str(), o);
  std::fclose(o);
  return 0;
}

// Reads a raw SoA event file (ndims x n doubles, n from the file size).
static bool read_events(const std::string& path, size_t nd, EventVector<kT, eT>*& out,
                        const std::vector<dimension<eT>*>& dims) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const size_t n = size_t(std::ftell(f)) / (8 * nd);
  std::fseek(f, 0, SEEK_SET);
  out = new EventVector<kT, eT>(dims, unsigned(n));
  const bool ok = std::fread(out->get_data(), 8, nd * n, f) == nd * n;
  std::fclose(f);
  return ok;
}

// The reference's fit (MIGRAD + HESSE through its fitter) of the events of a
// file on nthreads host threads: once from the truth (kernel text compiled
// by gcc on the way), then again from the truth with the kernels kept
// (fitter::fit refit), timed alone.
static int cmd_fitevents(const std::string& which, const std::string& path, unsigned nthreads) {
  compute_options copts;
  copts.llvm_nthreads = nthreads;
  copts.print_kernel = false;
  backendT backend(&copts);
  WorkloadT w = make_workload(which);
  EventVector<kT, eT>* data = nullptr;
  if (!read_events(path, w.dims.size(), data, w.dims)) return 2;
  std::vector<double> start;
  for (auto* p : w.params) start.push_back(p->get_value());
  fitter_options fopts = make_fit_opts(w);
  fitter<kT, eT, backendT, blockT> fit(&fopts, &backend);
  std::ostringstream sink;
  auto* old = std::cout.rdbuf(sink.rdbuf());
  auto t0 = std::chrono::steady_clock::now();
  fit.fit(w.pdf, w.params, data);
  auto t1 = std::chrono::steady_clock::now();
  std::vector<double> v, e;
  for (auto* p : w.params) {
    v.push_back(p->get_value());
    e.push_back(p->get_error());
  }
  for (size_t i = 0; i < start.size(); i++) {
    w.params[i]->set_value(start[i]);
    w.params[i]->set_start_value(start[i]);
  }
  auto t2 = std::chrono::steady_clock::now();
  fit.fit(w.pdf, w.params, data, true);
  auto t3 = std::chrono::steady_clock::now();
  std::cout.rdbuf(old);
  std::printf("{\"workload\":\"%s\",\"n\":%u,\"nthreads\":%u,\"events_fnv1a\":\"%016llx\",\"first_fit_ms\":%.3f,"
              "\"fit_ms\":%.3f,\"values\":%s,\"errors\":%s}\n",
              which.c_str(), data->nevents(), nthreads,
              (unsigned long long)fnv1a(data->get_data(), data->buffer_size()),
              std::chrono::duration<double, std::milli>(t1 - t0).count(),
              std::chrono::duration<double, std::milli>(t3 - t2).count(), jvec(v).c_str(), jvec(e).c_str());
  delete data;
  return 0;
}

// fitter::likelihood_and_gradient (the reference's NLL + gradient call,
// fitter.hh:1054-1151) over the events of a file on nthreads host threads,
// at the workload's truth: 3 untimed calls, then up to nevals calls or
// max_seconds of them, whichever ends first. One JSON line.
static int cmd_benchevents(const std::string& which, const std::string& path, unsigned nthreads, unsigned nevals,
                           double max_seconds) {
  compute_options copts;
  copts.llvm_nthreads = nthreads;
  copts.print_kernel = false;
  backendT backend(&copts);
  WorkloadT w = make_workload(which);
  EventVector<kT, eT>* data = nullptr;
  if (!read_events(path, w.dims.size(), data, w.dims)) return 2;
  fitter_options fopts = make_fit_opts(w);
  fopts.minuit_maxcalls = 1;
  fopts.minuit_maxiterations = 1;
  fopts.postrun_hesse = false;
  fitter<kT, eT, backendT, blockT> fit(&fopts, &backend);
  std::vector<double> truth;
  for (auto* p : w.params) truth.push_back(p->get_value());
  std::ostringstream sink;
  auto* old = std::cout.rdbuf(sink.rdbuf());
  fit.fit(w.pdf, w.params, data);  // builds the kernels and uploads the events
  for (size_t i = 0; i < truth.size(); i++) w.params[i]->set_value(truth[i]);
  const int npar = int(w.params.size());
  std::vector<double> grad(npar);
  double nll = 0.0;
  for (int i = 0; i < 3; i++) nll = fit.likelihood_and_gradient(npar, grad.data());
  auto t0 = std::chrono::steady_clock::now();
  unsigned done = 0;
  double s = 0.0;
  while (done < nevals) {
    nll = fit.likelihood_and_gradient(npar, grad.data());
    done++;
    s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (s >= max_seconds) break;
  }
  std::cout.rdbuf(old);
  std::printf("{\"workload\":\"%s\",\"nevents\":%u,\"nthreads\":%u,\"events_fnv1a\":\"%016llx\",\"nevals\":%u,"
              "\"seconds\":%.6f,\"evals_per_s\":%.6g,\"nll\":%.17g,\"grad\":%s}\n",
              which.c_str(), data->nevents(), nthreads,
              (unsigned long long)fnv1a(data->get_data(), data->buffer_size()), done, s, done / s, nll,
              jvec(grad).c_str());
  delete data;
  return 0;
}

int main(int argc, char** argv) {
  // MOREFIT_MINUIT_TOLERANCE: Minuit2's default tolerance for every fitter
  // this process makes (MIGRAD stops at EDM < 0.002 x tolerance); unset, the
  // Minuit2 default (0.01), as the reference's drivers run.
  if (const char* t = std::getenv("MOREFIT_MINUIT_TOLERANCE")) ROOT::Math::MinimizerOptions::SetDefaultTolerance(std::atof(t));
  install_capture();
  if (argc >= 5 && std::string(argv[1]) == "fitfile") return cmd_fitfile(argv[2], argv[3], argv[4]);
  if (argc >= 5 && std::string(argv[1]) == "fitevents")
    return cmd_fitevents(argv[2], argv[3], unsigned(std::stoul(argv[4])));
  if (argc >= 7 && std::string(argv[1]) == "benchevents")
    return cmd_benchevents(argv[2], argv[3], unsigned(std::stoul(argv[4])), unsigned(std::stoul(argv[5])),
                           std::stod(argv[6]));
  if (argc >= 5 && std::string(argv[1]) == "golden")
    return cmd_golden(argv[2], unsigned(std::stoul(argv[3])), argv[4], argc > 5 ? argv[5] : "");
  if (argc >= 6 && std::string(argv[1]) == "bench")
    return cmd_bench(argv[2], unsigned(std::stoul(argv[3])), unsigned(std::stoul(argv[4])),
                     unsigned(std::stoul(argv[5])));
  if (argc >= 8 && std::string(argv[1]) == "plot")
    return cmd_plot(argv[2], unsigned(std::stoul(argv[3])), argv[4], unsigned(std::stoul(argv[5])), argv[6], argv[7]);
  if (argc >= 7 && std::string(argv[1]) == "toys")
    return cmd_toys(argv[2], unsigned(std::stoul(argv[3])), std::stod(argv[4]), std::stod(argv[5]), argv[6],
                    argc > 7 ? std::stoull(argv[7]) : 229387429ULL);
  std::fprintf(stderr, "usage: refkit golden <mass|mass_w|cbpoly|pwave|spwave> <n> <out.json> [events.bin]\n"
                       "       refkit bench <mass|pwave|spwave> <n> <nthreads> <nevals>\n"
                       "       refkit toys <pwave> <ntoys> <mean events> <jitter> <out.json> [seed]\n"
                       "       refkit plot <workload> <n> <variable> <nbins> <out.py> <out.json>\n"
                       "       refkit fitfile <workload> <datasets.bin> <out.json>\n"
                       "       refkit fitevents <workload> <events.f64> <nthreads>\n"
                       "       refkit benchevents <workload> <events.f64> <nthreads> <nevals> <max seconds>\n");
  return 2;
}
