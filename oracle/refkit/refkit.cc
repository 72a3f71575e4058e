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
// Events come from generator::generate on the accelerator path with one
// xoshiro128++ stream seeded by Xoshiro128pp::setSeed(229387429)
// (random.hh:355-362, generator.hh:102-113), as in the reference drivers.
//
// Usage:
//   refkit golden <mass|pwave> <nevents> <out.json> [events.bin]
//   refkit bench  <mass|pwave> <nevents> <nthreads> <nevals>
//   refkit toys   <out.json> <ntoys> <mean> <seed>
#define MOREFIT_H 1  // keep graph.hh from pulling in the OpenCL/LLVM backends
#include <cassert>
#include <chrono>
#include <cmath>
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
#include "generator.hh"
#include "random.hh"

using namespace morefit;
typedef double kT;
typedef double eT;
typedef LLVMBackend backendT;
typedef LLVMBlock<kT, eT> blockT;

// ---- capture hooks: every parameter vector and Kahan result, per kernel ----
struct Capture {
  std::map<std::string, std::vector<double>> params, sums;
};
static Capture* g_capture = nullptr;
static void install_capture() {
  block_observer() = [](const std::string& kernel, const char* what, const std::vector<double>& v) {
    if (!g_capture) return;
    if (std::string(what) == "params")
      g_capture->params[kernel] = v;
    else
      g_capture->sums[kernel] = v;
  };
}

static std::string jstr(const std::string& s) {
  std::string o = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') o += '\\';
    o += c;
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

struct Workload {
  std::string name;
  std::vector<dimension<eT>*> dims;
  std::vector<parameter<eT>*> params;
  PDF<kT, eT>* pdf;
  bool optimize_dimensions;
};

static Workload make_workload(const std::string& which) {
  Workload w;
  w.name = which;
  if (which == "mass") {
    auto* m = new dimension<eT>("m", "m", 5000.0, 5600.0, false);
    auto* mb = new parameter<eT>("mb", "mb", 5280.0, 5200.0, 5400.0, 1.0, false);
    auto* sigma = new parameter<eT>("sigma", "sigma", 20.0, 5.0, 50.0, 0.5, false);
    auto* fsig = new parameter<eT>("fsig", "fsig", 0.3, 0.0, 1.0, 0.01, false);
    auto* alpha = new parameter<eT>("alpha", "alpha", -0.002, -0.01, 0.01, 0.0001, false);
    auto* gaus = new GaussianPDF<kT, eT>(m, mb, sigma);
    auto* ex = new ExponentialPDF<kT, eT>(m, alpha);
    w.pdf = new SumPDF<kT, eT>(gaus, ex, fsig);
    w.dims = {m};
    w.params = {mb, sigma, fsig, alpha};
    w.optimize_dimensions = false;
  } else if (which == "pwave") {
    auto* ctl = new dimension<eT>("ctl", "ctl", -1.0, 1.0, false);
    auto* ctk = new dimension<eT>("ctk", "ctk", -1.0, 1.0, false);
    auto* phi = new dimension<eT>("phi", "phi", -M_PI, +M_PI, false);
    auto* Fl = new parameter<eT>("Fl", "Fl", 0.70, 0.0, 1.0, 0.01, false);
    auto* S3 = new parameter<eT>("S3", "S3", -0.01, -1.0, 1.0, 0.01, false);
    auto* S4 = new parameter<eT>("S4", "S4", -0.15, -1.0, 1.0, 0.01, false);
    auto* S5 = new parameter<eT>("S5", "S5", -0.20, -1.0, 1.0, 0.01, false);
    auto* Afb = new parameter<eT>("Afb", "Afb", -0.10, -1.0, 1.0, 0.01, false);
    auto* S7 = new parameter<eT>("S7", "S7", 0.0, -1.0, 1.0, 0.01, false);
    auto* S8 = new parameter<eT>("S8", "S8", 0.0, -1.0, 1.0, 0.01, false);
    auto* S9 = new parameter<eT>("S9", "S9", 0.0, -1.0, 1.0, 0.01, false);
    w.pdf = new KstarmumuAngularPDF<kT, eT>(ctl, ctk, phi, Fl, S3, S4, S5, Afb, S7, S8, S9);
    w.dims = {ctl, ctk, phi};
    w.params = {Fl, S3, S4, S5, Afb, S7, S8, S9};
    w.optimize_dimensions = true;
  } else {
    std::fprintf(stderr, "unknown workload %s\n", which.c_str());
    std::exit(2);
  }
  return w;
}

static fitter_options make_fit_opts(const Workload& w) {
  fitter_options o;
  o.minimizer = fitter_options::minimizer_type::Minuit2;
  o.optimize_dimensions = w.optimize_dimensions;
  o.optimize_parameters = true;
  o.analytic_gradient = true;
  o.analytic_hessian = true;
  o.kahan_on_accelerator = true;
  o.print_level = 0;
  o.minuit_printlevel = 0;
  return o;
}

static void generate(Workload& w, backendT* backend, Xoshiro128pp* rnd, unsigned n, EventVector<kT, eT>& out) {
  generator_options gen_opts;
  gen_opts.rndtype = generator_options::randomization_type::on_accelerator;
  gen_opts.print_level = 0;
  generator<kT, eT, backendT, blockT> gen(&gen_opts, backend, rnd);
  gen.generate(n, w.pdf, w.params, out);
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
  Workload w = make_workload(which);
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
    for (int i = 0; i < npar; i++) d[i] = truth[i] + 0.5 * errors[i] * ((i % 2) ? -1.0 : 1.0);
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
    std::cout.rdbuf(old);
    g_capture = nullptr;
    pts += std::string(k ? "," : "") + "{\"params\":" + jvec(points[k]) + ",\"nll\":" + jnum(nll) +
           ",\"nll_from_grad_kernel\":" + jnum(nll2) + ",\"grad\":" + jvec(grad) + ",\"hessian\":" + jvec(h) +
           ",\"kernel_params\":{";
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
                   ",\"hessian_buffers\":" + jpairs(grab(log, "HESSIANBUFFER: ")) + ",\"fit\":{\"values\":" +
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
  Workload w = make_workload(which);
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

int main(int argc, char** argv) {
  install_capture();
  if (argc >= 5 && std::string(argv[1]) == "golden")
    return cmd_golden(argv[2], unsigned(std::stoul(argv[3])), argv[4], argc > 5 ? argv[5] : "");
  if (argc >= 6 && std::string(argv[1]) == "bench")
    return cmd_bench(argv[2], unsigned(std::stoul(argv[3])), unsigned(std::stoul(argv[4])),
                     unsigned(std::stoul(argv[5])));
  std::fprintf(stderr, "usage: refkit golden <mass|pwave> <n> <out.json> [events.bin]\n"
                       "       refkit bench <mass|pwave> <n> <nthreads> <nevals>\n");
  return 2;
}
