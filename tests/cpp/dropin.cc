// Drop-in check of include/compute_cuda.hh against the reference's unchanged
// fitter, generator and toystudy (compiled with the reference headers where
// they lie; built by tests/cpp/Makefile).
//
//   dropin lower <mass|pwave>   print the CUDA C the backend generates for every
//                               kernel the reference's fitter requests (works
//                               without a GPU: print_kernel output of the blocks)
//   dropin fit <mass|pwave> <n> generate n events on the GPU with the reference's
//                               generator and fit them with its fitter + Minuit2
//                               (needs a GB300)
#define MOREFIT_H 1
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <functional>
#include <iostream>
#include <sstream>
#include <string>

#include "graph.hh"
#include "eventvector.hh"
#include "parametervector.hh"
#include "pdf.hh"
#include "physicspdfs.hh"
#include "compute.hh"
#include "compute_cuda.hh"
#include "fitter.hh"
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
#include "toystudy.hh"

using namespace morefit;

template <typename kT>
static int run(const std::string& mode, const std::string& which, unsigned n) {
  typedef double eT;
  compute_options copts;
  copts.print_kernel = (mode == "lower");
  cuda_options cu;
  cu.quiet = (mode == "lower");
  CUDABackend backend(&copts, cu);
  std::vector<dimension<eT>*> dims;
  std::vector<parameter<eT>*> params;
  PDF<kT, eT>* pdf = nullptr;
  fitter_options fo;
  fo.minuit_printlevel = 0;
  fo.print_level = 0;
  if (which == "mass") {
    auto* m = new dimension<eT>("m", "m", 5000.0, 5600.0, false);
    auto* mb = new parameter<eT>("mb", "mb", 5280.0, 5200.0, 5400.0, 1.0, false);
    auto* sigma = new parameter<eT>("sigma", "sigma", 20.0, 5.0, 50.0, 0.5, false);
    auto* fsig = new parameter<eT>("fsig", "fsig", 0.3, 0.0, 1.0, 0.01, false);
    auto* alpha = new parameter<eT>("alpha", "alpha", -0.002, -0.01, 0.01, 0.0001, false);
    pdf = new SumPDF<kT, eT>(new GaussianPDF<kT, eT>(m, mb, sigma), new ExponentialPDF<kT, eT>(m, alpha), fsig);
    dims = {m};
    params = {mb, sigma, fsig, alpha};
    fo.optimize_dimensions = false;
  } else {
    auto* ctl = new dimension<eT>("ctl", "ctl", -1.0, 1.0, false);
    auto* ctk = new dimension<eT>("ctk", "ctk", -1.0, 1.0, false);
    auto* phi = new dimension<eT>("phi", "phi", -M_PI, +M_PI, false);
    const char* names[8] = {"Fl", "S3", "S4", "S5", "Afb", "S7", "S8", "S9"};
    const double truth[8] = {0.70, -0.01, -0.15, -0.20, -0.10, 0.0, 0.0, 0.0};
    for (int i = 0; i < 8; i++)
      params.push_back(new parameter<eT>(names[i], names[i], truth[i], i == 0 ? 0.0 : -1.0, 1.0, 0.01, false));
    pdf = new KstarmumuAngularPDF<kT, eT>(ctl, ctk, phi, params[0], params[1], params[2], params[3], params[4],
                                           params[5], params[6], params[7]);
    dims = {ctl, ctk, phi};
    fo.optimize_dimensions = true;
  }
  if (mode == "lower") {
    // make_kernels only reads the dimensions and event count of the data.
    EventVector<kT, eT> data(dims, 16);
    for (unsigned i = 0; i < 16 * dims.size(); i++) data.get_data()[i] = 0.5;
    fitter<kT, eT, CUDABackend, CUDABlock<kT, eT>> fit(&fo, &backend);
    fit.make_kernels(pdf, params, &data);
    return 0;
  }
  if (!backend.ok()) {
    std::printf("{\"skipped\":\"%s\"}\n", backend.error().c_str());
    return 0;
  }
  Xoshiro128pp rnd;
  rnd.setSeed(int64_t(229387429));
  generator_options go;
  go.print_level = 0;
  generator<kT, eT, CUDABackend, CUDABlock<kT, eT>> gen(&go, &backend, &rnd);
  EventVector<kT, eT> data(dims);
  gen.generate(n, pdf, params, data);
  fitter<kT, eT, CUDABackend, CUDABlock<kT, eT>> fit(&fo, &backend);
  auto t0 = std::chrono::steady_clock::now();
  fit.fit(pdf, params, &data);
  auto t1 = std::chrono::steady_clock::now();
  std::printf("{\"workload\":\"%s\",\"n\":%u,\"fit_ms\":%.3f,\"values\":[", which.c_str(), n,
              std::chrono::duration<double, std::milli>(t1 - t0).count());
  for (size_t i = 0; i < params.size(); i++) std::printf("%s%.17g", i ? "," : "", params[i]->get_value());
  std::printf("],\"errors\":[");
  for (size_t i = 0; i < params.size(); i++) std::printf("%s%.17g", i ? "," : "", params[i]->get_error());
  std::printf("]}\n");
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: dropin lower <mass|pwave> | dropin fit <mass|pwave> <n> [f32]\n");
    return 2;
  }
  std::string mode = argv[1], which = argv[2];
  unsigned n = argc > 3 ? unsigned(std::stoul(argv[3])) : 1000;
  bool f32 = argc > 4 && std::string(argv[4]) == "f32";
  return f32 ? run<float>(mode, which, n) : run<double>(mode, which, n);
}
