// Oracle kit: a CPU ComputeBlock that runs the reference's kernel text
// through the system C compiler.
//
// TEST INFRASTRUCTURE ONLY. This header is compiled together with the
// reference's own headers (graph.hh, pdf.hh, physicspdfs.hh, fitter.hh,
// generator.hh) and its vendored Minuit2, so that the reference's unchanged
// fitter and generator produce the golden vectors the CUDA backend is checked
// against. Nothing in the product links, loads or calls it.
//
// What it restates. The reference's CPU backend (include/compute_llvm.hh)
// wraps the expression strings that ComputeGraphNode::get_kernel() prints in
// a C function, compiles that with Clang/LLVM-17 ORC and runs it over
// contiguous event chunks. Clang/LLVM are absent here, so this block writes
// its own C wrapper around the same expression strings and compiles it with
// gcc into a shared object that it dlopen()s:
//   * compute kernel (compute_llvm.hh:535-750): per event, load every input
//     column `name = data[nevents*k + i]`, evaluate each graph, then either
//     store it (`output[nevents*j + i]`) or add it to a 4-lane interleaved
//     Kahan accumulator (lane = i % 4, compute_llvm.hh:556-568,656-709) whose
//     lanes are Kahan-combined in lane order at the end;
//   * thread split (compute_llvm.hh:751-932): nthreads contiguous chunks of
//     nevents/nthreads events (the last takes the remainder), per-chunk sums
//     Kahan-combined in chunk order (utils.hh:14-26);
//   * generate kernel (compute_llvm.hh:362-533): per thread one xoshiro128++
//     stream (seed rows from generator.hh:102-113), per event draw every
//     dimension as min + delta*u with min/delta printed "%.15e", evaluate the
//     normalised prob, accept when maxprob*u < prob.
// The class is named after the reference's LLVM backend types because
// generator.hh:102 selects the one-seed-per-thread layout by
// dynamic_cast<LLVMBackend*>.
#ifndef MOREFIT_ORACLE_GCC_BLOCK_HH
#define MOREFIT_ORACLE_GCC_BLOCK_HH

#include <dlfcn.h>
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "compute.hh"
#include "utils.hh"

namespace morefit {

class LLVMBackend : public ComputeBackend {
 public:
  explicit LLVMBackend(compute_options* opts) : ComputeBackend(opts) {}
};

// One recorded MakeComputeKernel call (used to dump kernel specs).
struct RecordedKernel {
  std::string name;
  std::vector<std::string> inputs, outputs, params, exprs;
  bool kahan = false;
  bool generate = false;
  std::vector<double> lo, hi;
  double maxprob = 0.0;
};

inline std::vector<RecordedKernel>& recorded_kernels() {
  static std::vector<RecordedKernel> r;
  return r;
}

// Observer of every parameter vector handed to a block ("params"), every
// Kahan result ("sums") and every output buffer ("outputs") read back, keyed
// by kernel name (golden capture).
using BlockObserver = std::function<void(const std::string&, const char*, const std::vector<double>&)>;
inline BlockObserver& block_observer() {
  static BlockObserver f;
  return f;
}

inline std::string oracle_workdir() {
  const char* d = std::getenv("MOREFIT_ORACLE_WORKDIR");
  std::string dir = d ? d : "/tmp/morefit_oracle_jit";
  std::string cmd = "mkdir -p " + dir;
  if (std::system(cmd.c_str()) != 0) std::abort();
  return dir;
}

inline void* compile_and_load(const std::string& name, const std::string& code) {
  static int counter = 0;
  std::string dir = oracle_workdir();
  std::string base = dir + "/" + name + "_" + std::to_string(::getpid()) + "_" + std::to_string(counter++);
  {
    std::ofstream f(base + ".c");
    f << code;
  }
#if defined(__x86_64__)
  const char* arch = "-march=x86-64-v3";  // compute_options::llvm_cpu default
#else
  const char* arch = "";
#endif
  std::string cmd = std::string("gcc -O3 -ffp-contract=off -fPIC -shared ") + arch + " -o " + base + ".so " +
                    base + ".c -lm";
  if (std::system(cmd.c_str()) != 0) {
    std::fprintf(stderr, "oracle: gcc failed for %s\n", base.c_str());
    std::abort();
  }
  void* h = dlopen((base + ".so").c_str(), RTLD_NOW | RTLD_LOCAL);
  if (!h) {
    std::fprintf(stderr, "oracle: dlopen failed: %s\n", dlerror());
    std::abort();
  }
  void* fn = dlsym(h, name.c_str());
  if (!fn) std::abort();
  return fn;
}

template <typename kernelT, typename evalT, typename seedT = uint32_t>
class LLVMBlock : public ComputeBlock<kernelT, evalT, seedT> {
  static_assert(std::is_same_v<kernelT, double> && std::is_same_v<evalT, double>,
                "oracle block is FP64 only");

 public:
  explicit LLVMBlock(LLVMBackend* backend) : backend_(backend) {}
  LLVMBlock(const LLVMBlock& o) : backend_(o.backend_) {}
  ~LLVMBlock() {
    if (holds_input_) delete[] input_;
    if (holds_output_) delete[] output_;
    delete[] params_;
    delete[] kahan_;
    delete[] seed_;
  }
  bool SetupInputBuffer(unsigned long nbytes) override {
    if (holds_input_) delete[] input_;
    input_ = new kernelT[nbytes / sizeof(kernelT) + 1];
    holds_input_ = true;
    return true;
  }
  bool SetupSeedBuffer(unsigned long nbytes) override {
    delete[] seed_;
    seed_ = new seedT[nbytes / sizeof(seedT) + 1];
    return true;
  }
  bool SetupInputBuffer(ComputeBlock<kernelT, evalT>* input, bool use_data_in = false) override {
    auto* other = dynamic_cast<LLVMBlock<kernelT, evalT>*>(input);
    if (holds_input_) delete[] input_;
    input_ = use_data_in ? other->input_ : other->output_;
    holds_input_ = false;
    return true;
  }
  bool SetupParameterBuffer(unsigned long nbytes) override {
    delete[] params_;
    params_ = new kernelT[nbytes / sizeof(kernelT) + 1];
    return true;
  }
  bool SetupOutputBuffer(unsigned long nbytes) override {
    if (holds_output_) delete[] output_;
    output_ = new kernelT[nbytes / sizeof(kernelT) + 1];
    holds_output_ = true;
    return true;
  }
  bool SetupKahanBuffer(unsigned long nbytes) override {
    delete[] kahan_;
    kahan_ = new evalT[nbytes / sizeof(evalT) + 1];
    return true;
  }
  bool SetNevents(int nevents, int nevents_padded = -1) override {
    nevents_ = nevents;
    nevents_padded_ = nevents_padded < 0 ? nevents : nevents_padded;
    return true;
  }
  bool CopyToInputBuffer(const EventVector<kernelT, evalT>& data) override {
    std::memcpy(input_, data.get_data(), data.buffer_size());
    return true;
  }
  bool CopyToSeedBuffer(const EventVector<seedT, evalT>& data) override {
    std::memcpy(seed_, data.get_data(), data.buffer_size());
    return true;
  }
  bool CopyToParameterBuffer(const std::vector<kernelT>& params) override {
    if (!params.empty()) std::memcpy(params_, params.data(), params.size() * sizeof(kernelT));
    if (block_observer()) block_observer()(name_, "params", params);
    return true;
  }
  bool CopyFromOutputBuffer(EventVector<kernelT, evalT>& data) override {
    std::memcpy(data.get_data(), output_, data.buffer_size());
    if (block_observer()) {
      const kernelT* o = reinterpret_cast<const kernelT*>(output_);
      block_observer()(name_, "outputs",
                       std::vector<double>(o, o + data.buffer_size() / sizeof(kernelT)));
    }
    return true;
  }
  bool CopyFromKahanBuffer(std::vector<evalT>& sums) override {
    std::memcpy(sums.data(), kahan_, sums.size() * sizeof(evalT));
    if (block_observer()) block_observer()(name_, "sums", sums);
    return true;
  }

  bool MakeGenerateKernel(std::string name, unsigned int nevents, std::vector<dimension<evalT>> input_signature,
                          std::vector<dimension<evalT>> output_signature, const std::vector<std::string>& params,
                          const std::vector<std::unique_ptr<ComputeGraphNode<kernelT, evalT>>>& graphs,
                          evalT maxprob = 1.0) override {
    generate_ = true;
    name_ = name;
    nevents_ = nevents_padded_ = nevents;
    RecordedKernel rec;
    rec.name = name;
    rec.generate = true;
    rec.params = params;
    for (auto& d : output_signature) {
      rec.outputs.push_back(d.get_name());
      rec.lo.push_back(d.get_min());
      rec.hi.push_back(d.get_max());
    }
    rec.exprs.push_back(graphs.at(0)->get_kernel());
    rec.maxprob = maxprob;
    recorded_kernels().push_back(rec);
    std::ostringstream c;
    c << "#include <math.h>\n#include <stdint.h>\n";
    c << "static inline uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }\n";
    c << "static inline double next_uniform(uint32_t* s) {\n"
         "  uint32_t r = rotl32(s[0] + s[3], 7) + s[0];\n"
         "  uint32_t t = s[1] << 9;\n"
         "  s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];\n"
         "  s[2] ^= t; s[3] = rotl32(s[3], 11);\n"
         "  return r * 2.3283064365386963e-10;\n}\n";
    c << "void " << name << "(unsigned nevents_padded, unsigned from, unsigned to, int tid, int nthr,"
      << " const uint32_t* seeds, double* output) {\n";
    c << "  uint32_t st[4];\n  for (int k = 0; k < 4; k++) st[k] = seeds[tid + k * nthr];\n";
    c << "  const double maxprob = " << fmt15(maxprob) << ";\n";
    for (auto& d : output_signature) c << "  double " << d.get_name() << ";\n";
    c << "  for (unsigned i = from; i < to; i++) {\n    for (;;) {\n";
    for (auto& d : output_signature)
      c << "      " << d.get_name() << " = " << fmt15(d.get_min()) << " + " << fmt15(d.get_max() - d.get_min())
        << " * next_uniform(st);\n";
    c << "      const double prob = " << graphs.at(0)->get_kernel() << ";\n";
    c << "      if (maxprob * next_uniform(st) < prob) {\n";
    for (size_t k = 0; k < output_signature.size(); k++)
      c << "        output[nevents_padded * " << k << "u + i] = " << output_signature[k].get_name() << ";\n";
    c << "        break;\n      }\n    }\n  }\n}\n";
    code_ = c.str();
    fn_ = compile_and_load(name, code_);
    return true;
  }

  bool MakeComputeKernel(std::string name, unsigned int nevents, std::vector<dimension<evalT>> input_signature,
                         std::vector<dimension<evalT>> output_signature, const std::vector<std::string>& params,
                         const std::vector<std::unique_ptr<ComputeGraphNode<kernelT, evalT>>>& graphs,
                         bool kahan_summation = false) override {
    generate_ = false;
    name_ = name;
    nevents_ = nevents_padded_ = nevents;
    kahan_summation_ = kahan_summation;
    nout_ = graphs.size();
    RecordedKernel rec;
    rec.name = name;
    rec.kahan = kahan_summation;
    for (auto& d : input_signature) rec.inputs.push_back(d.get_name());
    for (auto& d : output_signature) rec.outputs.push_back(d.get_name());
    rec.params = params;
    for (auto& g : graphs) rec.exprs.push_back(g->get_kernel());
    recorded_kernels().push_back(rec);

    const size_t M = graphs.size();
    std::ostringstream c;
    c << "#include <math.h>\n";
    c << "void " << name << "(unsigned nevents, unsigned from, unsigned to, const double* data,"
      << " double* output, const double* parameters, double* kahan) {\n";
    for (size_t k = 0; k < params.size(); k++)
      c << "  const double " << params[k] << " = parameters[" << k << "];\n";
    c << "  double lane_sum[" << 4 * M << "], lane_c[" << 4 * M << "];\n";
    c << "  for (int q = 0; q < " << 4 * M << "; q++) { lane_sum[q] = 0.0; lane_c[q] = 0.0; }\n";
    c << "  for (unsigned i = from; i < to; i++) {\n";
    for (size_t k = 0; k < input_signature.size(); k++)
      c << "    const double " << input_signature[k].get_name() << " = data[nevents * " << k << "u + i];\n";
    for (size_t j = 0; j < M; j++) c << "    const double r" << j << " = " << graphs[j]->get_kernel() << ";\n";
    c << "    if (kahan) {\n      const unsigned lane = i % 4u;\n";
    for (size_t j = 0; j < M; j++)
      c << "      { const unsigned q = " << 4 * j << "u + lane; const double y = r" << j
        << " - lane_c[q]; const double t = lane_sum[q] + y; lane_c[q] = (t - lane_sum[q]) - y; lane_sum[q] = t; }\n";
    c << "    } else {\n";
    for (size_t j = 0; j < M; j++) c << "      output[nevents * " << j << "u + i] = r" << j << ";\n";
    c << "    }\n  }\n";
    c << "  if (kahan) {\n    for (unsigned j = 0; j < " << M << "u; j++) {\n"
         "      double s = 0.0, cc = 0.0;\n"
         "      for (unsigned l = 0; l < 4u; l++) { const double y = lane_sum[4u * j + l] - cc; const double t = s + y;"
         " cc = (t - s) - y; s = t; }\n"
         "      kahan[j] = s;\n    }\n  }\n}\n";
    code_ = c.str();
    fn_ = compile_and_load(name, code_);
    return true;
  }

  bool SubmitKernel() override {
    const unsigned nthreads = backend_->opts_->llvm_nthreads > 0 ? backend_->opts_->llvm_nthreads : 1;
    if (generate_) {
      using gen_fn = void (*)(unsigned, unsigned, unsigned, int, int, const uint32_t*, double*);
      auto f = reinterpret_cast<gen_fn>(fn_);
      run_chunks(nthreads, [&](unsigned t, unsigned from, unsigned to) {
        f(nevents_padded_, from, to, int(t), int(nthreads), seed_, output_);
      });
      return true;
    }
    using cmp_fn = void (*)(unsigned, unsigned, unsigned, const double*, double*, const double*, double*);
    auto f = reinterpret_cast<cmp_fn>(fn_);
    if (!kahan_summation_) {
      run_chunks(nthreads, [&](unsigned, unsigned from, unsigned to) {
        f(nevents_, from, to, input_, output_, params_, nullptr);
      });
      return true;
    }
    std::vector<std::vector<double>> part(nthreads, std::vector<double>(nout_, 0.0));
    run_chunks(nthreads, [&](unsigned t, unsigned from, unsigned to) {
      f(nevents_, from, to, input_, output_, params_, part[t].data());
    });
    for (size_t j = 0; j < nout_; j++) {
      std::vector<double> col;
      for (unsigned t = 0; t < nthreads; t++) col.push_back(part[t][j]);
      kahan_[j] = kahan_summation<double, double>(col);
    }
    return true;
  }
  bool Finish() override { return true; }
  bool ProvidesKahan() override { return true; }

  const std::string& code() const { return code_; }

 private:
  static std::string fmt15(double v) {
    std::ostringstream s;
    s.precision(15);
    s << std::scientific << v;
    return s.str();
  }
  template <typename F>
  void run_chunks(unsigned nthreads, F&& body) {
    if (nthreads <= 1) {
      body(0u, 0u, nevents_);
      return;
    }
    std::vector<std::thread> ts;
    const unsigned size = nevents_ / nthreads;
    for (unsigned t = 0; t < nthreads; t++) {
      unsigned from = t * size, to = (t == nthreads - 1) ? nevents_ : t * size + size;
      ts.emplace_back([=, &body] { body(t, from, to); });
    }
    for (auto& th : ts) th.join();
  }

  LLVMBackend* backend_;
  std::string name_, code_;
  unsigned nevents_ = 0, nevents_padded_ = 0;
  size_t nout_ = 0;
  bool generate_ = false, kahan_summation_ = false;
  void* fn_ = nullptr;
  kernelT* input_ = nullptr;
  kernelT* output_ = nullptr;
  kernelT* params_ = nullptr;
  evalT* kahan_ = nullptr;
  seedT* seed_ = nullptr;
  bool holds_input_ = false, holds_output_ = false;
};

}  // namespace morefit

#endif
