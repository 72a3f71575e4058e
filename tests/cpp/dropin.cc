// Drop-in check of include/compute_cuda.hh against the reference's unchanged
// fitter, generator and Minuit2 (compiled from the reference sources by
// tests/cpp/Makefile; workloads from oracle/refkit/workloads.hh, the same
// models, parameters and fitter options as the golden vectors).
//
//   dropin lower <workload>                print the CUDA C the backend generates
//                                          for every kernel the reference's
//                                          fitter requests (no GPU needed)
//   dropin fit <workload> <events.f64> [f32|mixed]
//                                          fit the events of a raw SoA file
//                                          (ndims x n doubles) with the
//                                          reference's fitter + Minuit2 MIGRAD
//                                          and HESSE over CUDABlock<double> (or
//                                          CUDABlock<float> with f32, or
//                                          CUDABlock<double> with FP32 events
//                                          and arithmetic inside with mixed);
//                                          prints one JSON line
//   dropin genfit <workload> <n> [f32]     generate n events on the GPU with the
//                                          reference's generator (accelerator
//                                          partition, seed 229387429), then fit
//   dropin threads <workload> <coalesce|plain|serial> <f64|mixed> <events.f64>...
//                                          one host thread per event file, each
//                                          with its own fitter, CUDABlocks and
//                                          backend fitting that file, at once
//                                          (one thread after another: serial),
//                                          through a shared coalescer or not
//   dropin calls <workload> <events.f64> <count> [mixed] [launch]
//                                          latency of the fitter's FCN
//                                          evaluations after one fit: count
//                                          calls each of likelihood_and_gradient
//                                          (what MIGRAD calls), likelihood, and
//                                          MIGRAD's pattern (a gradient, two
//                                          values), at the fitted point, served
//                                          by the resident grid (default) or
//                                          with a launch per call (launch);
//                                          prints percentiles in microseconds
#define MOREFIT_H 1
#include <algorithm>
#include <atomic>
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <iostream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "graph.hh"
#include "eventvector.hh"
#include "parametervector.hh"
#include "pdf.hh"
#include "physicspdfs.hh"
#include "compute.hh"
#include "compute_cuda.hh"
#include "fitter.hh"
#include "Math/MinimizerOptions.h"
#include "random.hh"
// generator.hh selects its seeding by dynamic_cast<LLVMBackend*>; the CUDA
// backend takes the accelerator branch, so an empty LLVMBackend type suffices.
namespace morefit {
class LLVMBackend : public ComputeBackend {
 public:
  explicit LLVMBackend(compute_options* o) : ComputeBackend(o) {}
};
}  // namespace morefit
#include "generator.hh"
#include "workloads.hh"

using namespace morefit;

static uint64_t fnv1a(const void* p, size_t n) {
  const unsigned char* b = (const unsigned char*)p;
  uint64_t h = 1469598103934665603ULL;
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 1099511628211ULL;
  }
  return h;
}

static std::vector<double> read_events(const std::string& path, size_t ndims, unsigned& n) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", path.c_str());
    std::exit(2);
  }
  std::fseek(f, 0, SEEK_END);
  const long bytes = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  n = unsigned(size_t(bytes) / (8 * ndims));
  std::vector<double> v(ndims * size_t(n));
  if (std::fread(v.data(), 8, v.size(), f) != v.size()) {
    std::fprintf(stderr, "short read of %s\n", path.c_str());
    std::exit(2);
  }
  std::fclose(f);
  return v;
}

static std::string jvec(const std::vector<double>& v) {
  std::string o = "[";
  char b[64];
  for (size_t i = 0; i < v.size(); i++) {
    std::snprintf(b, sizeof b, "%s%.17g", i ? "," : "", v[i]);
    o += b;
  }
  return o + "]";
}

// "Hesse returns <status>" is the fitter's report of Minuit2's covariance status (fitter.hh:819-823).
static int cov_status_of(const std::string& log) {
  const std::string key = "Hesse returns ";
  size_t p = log.rfind(key);
  return p == std::string::npos ? -1 : std::atoi(log.c_str() + p + key.size());
}

struct FitResult {
  std::vector<double> values, errors;
  double first_ms = 0, warm_ms = 0;
  int cov_status = -1;
  bool ok = false;
  // |Newton step to the minimum of the fitted function| / error, per parameter,
  // at the fitted point (the fitter's own gradient and Hessian): how far MIGRAD
  // stopped from the minimum of the function it minimised
  std::vector<double> newton_sigma;
};

// Solves h x = g (h: n x n, row major) by Gaussian elimination with partial pivoting.
static std::vector<double> solve(std::vector<double> h, std::vector<double> g, size_t n) {
  for (size_t c = 0; c < n; c++) {
    size_t p = c;
    for (size_t r = c + 1; r < n; r++)
      if (std::fabs(h[r * n + c]) > std::fabs(h[p * n + c])) p = r;
    for (size_t k = 0; k < n; k++) std::swap(h[c * n + k], h[p * n + k]);
    std::swap(g[c], g[p]);
    for (size_t r = c + 1; r < n; r++) {
      const double f = h[r * n + c] / h[c * n + c];
      for (size_t k = c; k < n; k++) h[r * n + k] -= f * h[c * n + k];
      g[r] -= f * g[c];
    }
  }
  std::vector<double> x(n);
  for (size_t c = n; c-- > 0;) {
    double v = g[c];
    for (size_t k = c + 1; k < n; k++) v -= h[c * n + k] * x[k];
    x[c] = v / h[c * n + c];
  }
  return x;
}

// Discards what is written to it; no state, so several threads may write at once.
struct NullBuf : std::streambuf {
  int overflow(int c) override { return c; }
};

// One fit of `ev` (ndims x n doubles) with the reference's fitter over
// CUDABlock<kT>: first from the start values (this builds the kernels), then
// once more from the same start values with the kernels kept (refit), timed.
// With capture, the fitter's std::cout output is read for Minuit2's
// covariance status (one thread only; threads mode discards the output).
template <typename kT>
static FitResult fit_events(CUDABackend& backend, const std::string& which, const std::vector<double>& ev, unsigned n,
                            bool capture = true) {
  typedef double eT;
  Workload<kT, eT> w = make_workload<kT, eT>(which);
  const size_t nd = w.dims.size();
  EventVector<kT, eT> data(w.dims, n);
  for (size_t d = 0; d < nd; d++)
    for (unsigned i = 0; i < n; i++) data(i, d) = kT(ev[d * n + i]);
  std::vector<double> start;
  for (auto* p : w.params) start.push_back(p->get_value());
  fitter_options fo = make_fit_opts(w);
  fitter<kT, eT, CUDABackend, CUDABlock<kT, eT>> fit(&fo, &backend);
  FitResult r;
  std::ostringstream log;
  std::streambuf* old = capture ? std::cout.rdbuf(log.rdbuf()) : nullptr;
  auto t0 = std::chrono::steady_clock::now();
  r.ok = fit.fit(w.pdf, w.params, &data);
  auto t1 = std::chrono::steady_clock::now();
  if (capture) r.cov_status = cov_status_of(log.str());
  for (auto* p : w.params) {
    r.values.push_back(p->get_value());
    r.errors.push_back(p->get_error());
  }
  if (capture) {
    const int np = int(w.params.size());
    std::vector<double> g(np), h(size_t(np) * np);
    fit.likelihood_and_gradient(np, g.data());
    fit.hessian(np, h.data());
    const std::vector<double> step = solve(h, g, size_t(np));
    for (int i = 0; i < np; i++) r.newton_sigma.push_back(std::fabs(step[i]) / r.errors[i]);
  }
  for (size_t i = 0; i < start.size(); i++) {
    w.params[i]->set_value(start[i]);
    w.params[i]->set_start_value(start[i]);
  }
  auto t2 = std::chrono::steady_clock::now();
  fit.fit(w.pdf, w.params, &data, true);
  auto t3 = std::chrono::steady_clock::now();
  if (capture) std::cout.rdbuf(old);
  r.first_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  r.warm_ms = std::chrono::duration<double, std::milli>(t3 - t2).count();
  return r;
}

static void print_fit(const std::string& which, unsigned n, const char* prec, uint64_t hash, const FitResult& r,
                      const char* extra = "") {
  std::printf("{\"workload\":\"%s\",\"n\":%u,\"kernelT\":\"%s\",\"events_fnv1a\":\"%016llx\",\"ok\":%s,"
              "\"cov_status\":%d,\"first_fit_ms\":%.3f,\"fit_ms\":%.3f,\"values\":%s,\"errors\":%s,"
              "\"newton_sigma\":%s%s}\n",
              which.c_str(), n, prec, (unsigned long long)hash, r.ok ? "true" : "false", r.cov_status, r.first_ms,
              r.warm_ms, jvec(r.values).c_str(), jvec(r.errors).c_str(), jvec(r.newton_sigma).c_str(), extra);
}

template <typename kT>
static int cmd_lower(const std::string& which) {
  typedef double eT;
  compute_options copts;
  copts.print_kernel = true;
  cuda_options cu;
  cu.quiet = true;
  CUDABackend backend(&copts, cu);
  Workload<kT, eT> w = make_workload<kT, eT>(which);
  // make_kernels only reads the dimensions and event count of the data.
  EventVector<kT, eT> data(w.dims, 16);
  for (unsigned i = 0; i < 16 * w.dims.size(); i++) data.get_data()[i] = 0.5;
  fitter_options fo = make_fit_opts(w);
  fitter<kT, eT, CUDABackend, CUDABlock<kT, eT>> fit(&fo, &backend);
  fit.make_kernels(w.pdf, w.params, &data);
  return 0;
}

template <typename kT>
static int cmd_fit(const std::string& which, const std::string& path, const char* prec, bool mixed = false) {
  compute_options copts;
  cuda_options cu;
  cu.mixed_precision = mixed;
  CUDABackend backend(&copts, cu);
  if (!backend.ok()) {
    std::printf("{\"skipped\":\"%s\"}\n", backend.error().c_str());
    return 3;
  }
  Workload<double, double> w0 = make_workload<double, double>(which);
  unsigned n = 0;
  std::vector<double> ev = read_events(path, w0.dims.size(), n);
  const uint64_t h = fnv1a(ev.data(), ev.size() * sizeof(double));
  FitResult r = fit_events<kT>(backend, which, ev, n);
  print_fit(which, n, prec, h, r);
  return r.ok ? 0 : 1;
}

template <typename kT>
static int cmd_genfit(const std::string& which, unsigned n, const char* prec) {
  typedef double eT;
  compute_options copts;
  CUDABackend backend(&copts);
  if (!backend.ok()) {
    std::printf("{\"skipped\":\"%s\"}\n", backend.error().c_str());
    return 3;
  }
  // the reference's generator over CUDABlock: accelerator partition over
  // compute_options::opencl_max_generator_workitems threads (generator.hh:102-175)
  Workload<kT, eT> w = make_workload<kT, eT>(which);
  Xoshiro128pp rnd;
  rnd.setSeed(int64_t(229387429));
  generator_options go;
  go.rndtype = generator_options::randomization_type::on_accelerator;
  go.print_level = 0;
  EventVector<kT, eT> data(w.dims);
  auto t0 = std::chrono::steady_clock::now();
  {
    generator<kT, eT, CUDABackend, CUDABlock<kT, eT>> gen(&go, &backend, &rnd);
    std::ostringstream log;
    auto* old = std::cout.rdbuf(log.rdbuf());
    gen.generate(n, w.pdf, w.params, data);
    std::cout.rdbuf(old);
  }
  auto t1 = std::chrono::steady_clock::now();
  const size_t nd = w.dims.size();
  n = data.nevents();
  std::vector<double> ev(nd * size_t(n));
  for (size_t d = 0; d < nd; d++)
    for (unsigned i = 0; i < n; i++) ev[d * n + i] = double(data(i, d));
  const uint64_t h = fnv1a(ev.data(), ev.size() * sizeof(double));
  FitResult r = fit_events<kT>(backend, which, ev, n);
  char extra[96];
  std::snprintf(extra, sizeof extra, ",\"generate_ms\":%.3f",
                std::chrono::duration<double, std::milli>(t1 - t0).count());
  print_fit(which, n, prec, h, r, extra);
  return r.ok ? 0 : 1;
}

// Per-call latency of the reference fitter's evaluations over CUDABlock: one
// fit builds the kernels and uploads the events, then each timed call is one
// FCN evaluation as Minuit2 makes it (hoisted parameter buffers on the host,
// CopyToParameterBuffer, SubmitKernel, Finish, CopyFromKahanBuffer).
static int cmd_calls(const std::string& which, const std::string& path, int count, bool mixed, bool launch) {
  typedef double kT;
  typedef double eT;
  compute_options copts;
  cuda_options cu;
  cu.mixed_precision = mixed;
  if (launch) cu.resident_idle_us = 0;
  CUDABackend backend(&copts, cu);
  if (!backend.ok()) {
    std::printf("{\"skipped\":\"%s\"}\n", backend.error().c_str());
    return 3;
  }
  Workload<kT, eT> w = make_workload<kT, eT>(which);
  unsigned n = 0;
  std::vector<double> ev = read_events(path, w.dims.size(), n);
  const size_t nd = w.dims.size();
  EventVector<kT, eT> data(w.dims, n);
  for (size_t d = 0; d < nd; d++)
    for (unsigned i = 0; i < n; i++) data(i, d) = ev[d * n + i];
  fitter_options fo = make_fit_opts(w);
  fitter<kT, eT, CUDABackend, CUDABlock<kT, eT>> fit(&fo, &backend);
  std::ostringstream log;
  std::streambuf* old = std::cout.rdbuf(log.rdbuf());
  const bool ok = fit.fit(w.pdf, w.params, &data);
  std::cout.rdbuf(old);
  const int np = int(w.params.size());
  std::vector<double> g(np);
  auto pct = [](std::vector<double> t) {
    std::sort(t.begin(), t.end());
    char b[160];
    std::snprintf(b, sizeof b, "{\"p10\":%.3f,\"p50\":%.3f,\"p90\":%.3f}", t[t.size() / 10], t[t.size() / 2],
                  t[t.size() * 9 / 10]);
    return std::string(b);
  };
  std::vector<double> tg, tl;
  double sink = 0.0;
  // The fit's calls start the resident module's build on a background thread
  // (an NVRTC compile of a second or two when the kernel cache is cold);
  // time the steady state, once it is ready (or given up), as a long fit sees it.
  int build_state = -1;
  if (!launch) {
    const auto until = std::chrono::steady_clock::now() + std::chrono::seconds(30);
    do {
      sink += fit.likelihood();
      mf_context_resident_stats(backend.context(), &build_state, nullptr, nullptr, nullptr);
      if (build_state >= 2) break;
      std::this_thread::sleep_for(std::chrono::milliseconds(2));
    } while (std::chrono::steady_clock::now() < until);
  }
  for (int i = 0; i < count + 50; i++) {
    auto t0 = std::chrono::steady_clock::now();
    sink += fit.likelihood_and_gradient(np, g.data());
    auto t1 = std::chrono::steady_clock::now();
    if (i >= 50) tg.push_back(std::chrono::duration<double, std::micro>(t1 - t0).count());
  }
  for (int i = 0; i < count + 50; i++) {
    auto t0 = std::chrono::steady_clock::now();
    sink += fit.likelihood();
    auto t1 = std::chrono::steady_clock::now();
    if (i >= 50) tl.push_back(std::chrono::duration<double, std::micro>(t1 - t0).count());
  }
  // MIGRAD's pattern: a gradient, then line-search values
  std::vector<double> ta;
  for (int i = 0; i < count + 50; i++) {
    auto t0 = std::chrono::steady_clock::now();
    sink += fit.likelihood_and_gradient(np, g.data());
    sink += fit.likelihood();
    sink += fit.likelihood();
    auto t1 = std::chrono::steady_clock::now();
    if (i >= 50) ta.push_back(std::chrono::duration<double, std::micro>(t1 - t0).count() / 3.0);
  }
  int state = -1, blocks = 0;
  uint64_t grids = 0, served = 0;
  mf_context_resident_stats(backend.context(), &state, &grids, &served, &blocks);
  std::printf("{\"workload\":\"%s\",\"n\":%u,\"mixed\":%s,\"resident\":%s,\"fit_ok\":%s,\"count\":%d,"
              "\"likelihood_and_gradient_us\":%s,\"likelihood_us\":%s,\"migrad_pattern_us_per_call\":%s,"
              "\"resident_stats\":{\"state\":%d,\"grids\":%llu,\"served\":%llu,\"blocks\":%d},"
              "\"finite\":%s}\n",
              which.c_str(), n, mixed ? "true" : "false", launch ? "false" : "true", ok ? "true" : "false", count,
              pct(tg).c_str(), pct(tl).c_str(), pct(ta).c_str(), state, (unsigned long long)grids,
              (unsigned long long)served, blocks, std::isfinite(sink) ? "true" : "false");
  return ok ? 0 : 1;
}

// Several host threads, each with its own fitter, CUDABlocks and backend
// (context), fitting its own dataset: one fitter per host thread, the
// reference's threading model. mode "coalesce": every backend routes its
// synchronous evaluations through one shared coalescer; "plain": no
// coalescer (each context launches on its own stream); "serial": one thread
// fits the datasets one after another. Each fit is timed from the start of
// the thread's work on it (kernel builds, upload, MIGRAD + HESSE).
static int cmd_threads(const std::string& which, const std::string& mode, bool mixed,
                       const std::vector<std::string>& files) {
  Workload<double, double> w0 = make_workload<double, double>(which);
  const size_t T = files.size();
  std::vector<std::vector<double>> ev(T);
  std::vector<unsigned> ns(T);
  for (size_t t = 0; t < T; t++) ev[t] = read_events(files[t], w0.dims.size(), ns[t]);
  mf_coalescer* co = nullptr;
  if (mode == "coalesce" && mf_coalescer_create(0, 0, 30, &co) != MF_OK) {
    std::printf("{\"skipped\":\"%s\"}\n", mf_last_error());
    return 3;
  }
  std::vector<FitResult> res(T);
  std::vector<double> latency(T);
  std::atomic<bool> failed{false};
  NullBuf null;
  auto* old = std::cout.rdbuf(&null);
  auto t0 = std::chrono::steady_clock::now();
  auto one = [&](size_t t) {
    compute_options copts;
    cuda_options cu;
    cu.mixed_precision = mixed;
    cu.coalescer = co;
    cu.quiet = true;
    CUDABackend backend(&copts, cu);
    if (!backend.ok()) {
      failed = true;
      return;
    }
    auto a = std::chrono::steady_clock::now();
    res[t] = fit_events<double>(backend, which, ev[t], ns[t], false);
    latency[t] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
  };
  if (mode == "serial") {
    for (size_t t = 0; t < T; t++) one(t);
  } else {
    std::vector<std::thread> th;
    for (size_t t = 0; t < T; t++) th.emplace_back(one, t);
    for (auto& x : th) x.join();
  }
  auto t1 = std::chrono::steady_clock::now();
  std::cout.rdbuf(old);
  uint64_t ticks = 0, evals = 0;
  uint32_t maxb = 0;
  if (co) {
    mf_coalescer_stats(co, &ticks, &evals, &maxb);
    mf_coalescer_destroy(co);
  }
  if (failed) {
    std::printf("{\"skipped\":\"no CUDA context\"}\n");
    return 3;
  }
  std::printf("{\"workload\":\"%s\",\"mode\":\"%s\",\"mixed\":%s,\"nthreads\":%zu,\"wall_ms\":%.3f,"
              "\"coalescer\":{\"ticks\":%llu,\"evaluations\":%llu,\"max_batch\":%u},\"fits\":[",
              which.c_str(), mode.c_str(), mixed ? "true" : "false", T,
              std::chrono::duration<double, std::milli>(t1 - t0).count(), (unsigned long long)ticks,
              (unsigned long long)evals, maxb);
  bool ok = true;
  for (size_t t = 0; t < T; t++) {
    ok = ok && res[t].ok;
    std::printf("%s{\"n\":%u,\"ok\":%s,\"latency_ms\":%.3f,\"fit_ms\":%.3f,\"values\":%s,\"errors\":%s}",
                t ? "," : "", ns[t], res[t].ok ? "true" : "false", latency[t], res[t].warm_ms,
                jvec(res[t].values).c_str(), jvec(res[t].errors).c_str());
  }
  std::printf("]}\n");
  return ok ? 0 : 1;
}

int main(int argc, char** argv) {
  // MOREFIT_MINUIT_TOLERANCE: Minuit2's default tolerance for every fitter
  // this process makes (MIGRAD stops at EDM < 0.002 x tolerance); unset, the
  // Minuit2 default (0.01), as the reference's drivers run.
  if (const char* t = std::getenv("MOREFIT_MINUIT_TOLERANCE")) ROOT::Math::MinimizerOptions::SetDefaultTolerance(std::atof(t));
  const std::string usage =
      "usage: dropin lower <workload> | dropin fit <workload> <events.f64> [f32|mixed] | "
      "dropin genfit <workload> <n> [f32] | "
      "dropin threads <workload> <coalesce|plain|serial> <f64|mixed> <events.f64>... | "
      "dropin calls <workload> <events.f64> <count> [mixed] [launch]\n";
  if (argc < 3) {
    std::fprintf(stderr, "%s", usage.c_str());
    return 2;
  }
  const std::string mode = argv[1], which = argv[2];
  auto is_f32 = [&](int i) { return argc > i && std::string(argv[i]) == "f32"; };
  if (mode == "lower") return is_f32(3) ? cmd_lower<float>(which) : cmd_lower<double>(which);
  if (mode == "fit" && argc >= 4) {
    if (argc > 4 && std::string(argv[4]) == "mixed") return cmd_fit<double>(which, argv[3], "double, mixed", true);
    return is_f32(4) ? cmd_fit<float>(which, argv[3], "float") : cmd_fit<double>(which, argv[3], "double");
  }
  if (mode == "genfit" && argc >= 4) {
    const unsigned n = unsigned(std::stoul(argv[3]));
    return is_f32(4) ? cmd_genfit<float>(which, n, "float") : cmd_genfit<double>(which, n, "double");
  }
  if (mode == "calls" && argc >= 5) {
    bool mixed = false, launch = false;
    for (int i = 5; i < argc; i++) {
      mixed = mixed || std::string(argv[i]) == "mixed";
      launch = launch || std::string(argv[i]) == "launch";
    }
    return cmd_calls(which, argv[3], std::atoi(argv[4]), mixed, launch);
  }
  if (mode == "threads" && argc >= 6) {
    std::vector<std::string> files(argv + 5, argv + argc);
    return cmd_threads(which, argv[3], std::string(argv[4]) == "mixed", files);
  }
  std::fprintf(stderr, "%s", usage.c_str());
  return 2;
}
