/**
 * compute_cuda.hh — GB300 (sm_103a) compute backend for MoreFit.
 *
 * Drop-in implementation of the reference's backend interface,
 * morefit::ComputeBackend and morefit::ComputeBlock<kernelT, evalT, seedT>
 * (reference include/compute.hh:98-149), on top of the C ABI in
 * morefit_cuda.h. Use it as the backendT / computeT template arguments of the
 * reference's unchanged fitter, generator and toystudy:
 *
 *   morefit::CUDABackend backend(&compute_opts);
 *   morefit::fitter<double, double, morefit::CUDABackend,
 *                   morefit::CUDABlock<double, double>> fit(&fit_opts, &backend);
 *
 * kernelT = double gives the plain FP64 path; kernelT = float gives the
 * reference's mixed-precision interface (FP32 event columns and per-event
 * arithmetic, FP64 sums; evalT stays double). With kernelT = float the
 * reference's fitter hands every parameter and hoisted parameter buffer to
 * the block rounded to FP32 (fitter.hh:1059-1073), each rounded on its own,
 * so the likelihood it minimises jumps by about N * 6e-8 whenever one of
 * them crosses an FP32 boundary (~0.03 at 1M events): more than MIGRAD's
 * convergence test tolerates. cuda_options::mixed_precision keeps kernelT =
 * double at the interface (FP64 parameters) and stores and computes the
 * events in FP32 inside the block: the function stays smooth in the
 * parameters and fits agree with FP64 ones to ~1e-5 sigma.
 *
 * Mapping of the interface (reference line -> this class):
 *  - MakeComputeKernel (compute.hh:143) hands the ComputeGraphNode
 *    get_kernel() strings to mf_kernel_build, which shares subexpressions
 *    across all outputs, lowers them to CUDA C and compiles them with NVRTC;
 *    kahan_summation selects a fused reduce kernel (one launch: per-thread
 *    partials, warp/block tree, fixed-order compensated combine of the block
 *    partials) instead of the OpenCL backend's separate multi-pass Kahan
 *    reduction (compute_opencl.hh:807-991).
 *  - MakeGenerateKernel (compute.hh:140) builds the accept-reject kernel with
 *    the accelerator work partition (compute_opencl.hh:437-445,505-515).
 *  - Buffers are device structure-of-arrays blocks whose column stride is
 *    padded internally (MF_COLUMN_ALIGN), so required_padding() is 0 and host
 *    EventVectors stay unpadded. SetupInputBuffer(block, use_data_in) shares
 *    the other block's device columns, as the reference's chained blocks do
 *    (compute_llvm.hh:290-301, compute_opencl.hh:299-315).
 *  - Every failure is reported through the bool return and last_error() and
 *    printed once; nothing asserts or aborts (the reference asserts,
 *    compute_opencl.hh:279-283).
 *
 * Include after the reference's compute.hh (this header includes it).
 */
#ifndef MOREFIT_COMPUTE_CUDA_HH
#define MOREFIT_COMPUTE_CUDA_HH

#include <cstdint>
#include <cstring>
#include <iostream>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "compute.hh"
#include "morefit_cuda.h"

namespace morefit {

struct cuda_options {
  int device = 0;
  uint64_t hbm_budget_bytes = 0;  // 0 = no cap
  bool quiet = false;             // do not print failures to std::cerr
  // CUDABlock<double>: FP32 event columns and per-event arithmetic behind the
  // FP64 interface (FP64 parameters, sums and Minuit2 covariance)
  bool mixed_precision = false;
  // Route every synchronous evaluation of this backend's blocks through a
  // coalescer shared with other threads' backends (mf_coalescer_create);
  // not owned, must outlive the backend.
  mf_coalescer* coalescer = nullptr;
  // Serve the synchronous evaluations of the two most used kernels (a fit's
  // likelihood and likelihood + gradient) from a resident grid that leaves
  // after this many microseconds without requests (mf_context_set_resident);
  // 0 = a launch per evaluation. Sums are bit-identical either way.
  uint32_t resident_idle_us = 2000;
};

class CUDABackend : public ComputeBackend {
 public:
  explicit CUDABackend(compute_options* opts, cuda_options copts = cuda_options()) : ComputeBackend(opts), copts_(copts) {
    if (mf_context_create(copts_.device, copts_.hbm_budget_bytes, &ctx_) != MF_OK) {
      error_ = mf_last_error();
      ctx_ = nullptr;
      if (!copts_.quiet) std::cerr << "CUDABackend: " << error_ << std::endl;
      return;
    }
    if (copts_.coalescer && mf_context_set_coalescer(ctx_, copts_.coalescer) != MF_OK) {
      error_ = mf_last_error();
      mf_context_destroy(ctx_);
      ctx_ = nullptr;
      if (!copts_.quiet) std::cerr << "CUDABackend: " << error_ << std::endl;
      return;
    }
    // unsupported on the device: evaluations launch as usual
    if (!copts_.coalescer && copts_.resident_idle_us) mf_context_set_resident(ctx_, copts_.resident_idle_us);
  }
  ~CUDABackend() {
    if (!ctx_) return;
    if (copts_.coalescer) mf_context_set_coalescer(ctx_, nullptr);
    mf_context_destroy(ctx_);
  }
  CUDABackend(const CUDABackend&) = delete;
  CUDABackend& operator=(const CUDABackend&) = delete;
  virtual int required_padding() const override { return 0; }
  bool ok() const { return ctx_ != nullptr; }
  const std::string& error() const { return error_; }
  mf_context* context() const { return ctx_; }
  const cuda_options& cuda_opts() const { return copts_; }

 private:
  cuda_options copts_;
  mf_context* ctx_ = nullptr;
  std::string error_;
};

namespace cuda_detail {

// A device SoA block: ncols columns of n events with a padded column stride.
struct Columns {
  mf_context* ctx = nullptr;
  int elem = MF_F64;
  mf_buffer* buf = nullptr;
  uint32_t ncols = 0;
  uint64_t n = 0, stride = 0;
  explicit Columns(mf_context* c, int e) : ctx(c), elem(e) {}
  ~Columns() {
    if (buf) mf_buffer_free(buf);
  }
  size_t itemsize() const { return elem == MF_F32 ? 4 : 8; }
  int ensure(uint32_t cols, uint64_t events) {
    const uint64_t s = mf_column_stride(events);
    const uint64_t need = uint64_t(cols ? cols : 1) * s * itemsize();
    if (!buf || mf_buffer_size(buf) < need) {
      if (buf) mf_buffer_free(buf);
      buf = nullptr;
      int rc = mf_buffer_alloc(ctx, need, &buf);
      if (rc != MF_OK) return rc;
    }
    ncols = cols;
    n = events;
    stride = s;
    return MF_OK;
  }
};

}  // namespace cuda_detail

template <typename kernelT, typename evalT, typename seedT = uint32_t>
class CUDABlock : public ComputeBlock<kernelT, evalT, seedT> {
  static_assert(std::is_same_v<kernelT, double> || std::is_same_v<kernelT, float>,
                "CUDABlock supports kernelT = double (FP64) or float (mixed precision)");
  static_assert(std::is_same_v<seedT, uint32_t>, "the accelerator generator uses xoshiro128++ (uint32_t seeds)");
  using Columns = cuda_detail::Columns;

 public:
  explicit CUDABlock(CUDABackend* backend)
      : backend_(backend),
        kElem(std::is_same_v<kernelT, float> || (backend && backend->cuda_opts().mixed_precision) ? MF_F32 : MF_F64) {}
  ~CUDABlock() {
    if (kernel_) mf_kernel_free(kernel_);
  }

  // ---- buffers (compute.hh:114-128) ----
  virtual bool SetupInputBuffer(unsigned long int) override {
    if (!ready()) return false;
    input_ = std::make_shared<Columns>(backend_->context(), kElem);  // allocated on CopyToInputBuffer
    return true;
  }
  virtual bool SetupSeedBuffer(unsigned long int) override { return ready(); }
  virtual bool SetupInputBuffer(ComputeBlock<kernelT, evalT>* input, bool use_data_in = false) override {
    auto* other = dynamic_cast<CUDABlock<kernelT, evalT, seedT>*>(input);
    if (!other) return fail("SetupInputBuffer: the other block is not a CUDABlock of the same types");
    if (!ready()) return false;
    if (use_data_in) {
      if (!other->input_) other->input_ = std::make_shared<Columns>(backend_->context(), kElem);
      input_ = other->input_;
    } else {
      if (!other->output_) other->output_ = std::make_shared<Columns>(backend_->context(), kElem);
      input_ = other->output_;
    }
    return true;
  }
  virtual bool SetupParameterBuffer(unsigned long int nbytes) override {
    params_.reserve(nbytes / sizeof(kernelT));
    return ready();
  }
  virtual bool SetupOutputBuffer(unsigned long int) override {
    if (!ready()) return false;
    if (!output_) output_ = std::make_shared<Columns>(backend_->context(), kElem);  // kept: chained blocks share it
    return true;
  }
  virtual bool SetupKahanBuffer(unsigned long int nbytes) override {
    kahan_.assign(nbytes / sizeof(evalT), evalT(0));
    return true;
  }
  virtual bool SetNevents(int nevents, int nevents_padded = -1) override {
    nevents_ = nevents < 0 ? 0u : unsigned(nevents);
    return true;
  }

  // ---- copies (compute.hh:130-138) ----
  virtual bool CopyToInputBuffer(const EventVector<kernelT, evalT>& data) override {
    if (!ready()) return false;
    if (!input_) input_ = std::make_shared<Columns>(backend_->context(), kElem);
    const uint32_t ncols = data.ndimensions();
    const uint64_t n = data.nevents();
    if (check(input_->ensure(ncols, n))) return false;
    if constexpr (std::is_same_v<kernelT, double>)
      if (kElem == MF_F32)  // mixed precision behind the FP64 interface
        return !check(mf_events_upload_f64_as(input_->buf, MF_F32, data.get_data(), ncols, n, data.nevents_padded(),
                                              input_->stride));
    return !check(mf_events_upload(input_->buf, kElem, data.get_data(), ncols, n, data.nevents_padded(),
                                   input_->stride));
  }
  virtual bool CopyToSeedBuffer(const EventVector<seedT, evalT>& data) override {
    seed_rows_ = data.nevents_padded();
    seeds_.assign(data.get_data(), data.get_data() + size_t(4) * seed_rows_);
    return true;
  }
  virtual bool CopyToParameterBuffer(const std::vector<kernelT>& params) override {
    params_.assign(params.begin(), params.end());
    return true;
  }
  virtual bool CopyFromOutputBuffer(EventVector<kernelT, evalT>& data) override {
    if (!output_ || !output_->buf) return fail("CopyFromOutputBuffer: no output on the device");
    const uint32_t ncols = std::min<uint32_t>(data.ndimensions(), output_->ncols);
    const uint64_t n = std::min<uint64_t>(data.nevents(), output_->n);
    if constexpr (std::is_same_v<kernelT, double>)
      if (kElem == MF_F32) {  // FP32 columns into an FP64 EventVector
        std::vector<float> tmp(size_t(ncols) * n);
        if (check(mf_events_download(output_->buf, MF_F32, tmp.data(), ncols, n, n, output_->stride))) return false;
        const uint64_t hs = data.nevents_padded();
        for (uint32_t c = 0; c < ncols; c++)
          for (uint64_t i = 0; i < n; i++) data.get_data()[c * hs + i] = double(tmp[c * n + i]);
        return true;
      }
    return !check(mf_events_download(output_->buf, kElem, data.get_data(), ncols, n, data.nevents_padded(),
                                     output_->stride));
  }
  virtual bool CopyFromKahanBuffer(std::vector<evalT>& sums) override {
    const size_t m = std::min(sums.size(), kahan_.size());
    std::copy(kahan_.begin(), kahan_.begin() + m, sums.begin());
    return m == sums.size();
  }

  // ---- kernels (compute.hh:140-148) ----
  virtual bool MakeGenerateKernel(std::string name, unsigned int nevents, std::vector<dimension<evalT>> input_signature,
                                  std::vector<dimension<evalT>> output_signature, const std::vector<std::string>& params,
                                  const std::vector<std::unique_ptr<ComputeGraphNode<kernelT, evalT>>>& graphs,
                                  evalT maxprob = 1.0) override {
    if (!ready()) return false;
    if (graphs.size() != 1) return fail("MakeGenerateKernel: exactly one density graph expected");
    std::vector<std::string> dims;
    std::vector<double> lo, hi;
    for (auto& d : output_signature) {
      dims.push_back(d.get_name());
      lo.push_back(double(d.get_min()));
      hi.push_back(double(d.get_max()));
    }
    std::vector<std::string> exprs{graphs[0]->get_kernel()};
    kind_ = MF_KERNEL_GENERATE;
    nevents_ = nevents;
    ndims_ = uint32_t(dims.size());
    return build(name, {}, params, exprs, &dims, &lo, &hi, double(maxprob));
  }

  virtual bool MakeComputeKernel(std::string name, unsigned int nevents, std::vector<dimension<evalT>> input_signature,
                                 std::vector<dimension<evalT>> output_signature, const std::vector<std::string>& params,
                                 const std::vector<std::unique_ptr<ComputeGraphNode<kernelT, evalT>>>& graphs,
                                 bool kahan_summation = false) override {
    if (output_signature.size() != graphs.size())
      return fail("MakeComputeKernel: output signature and graphs differ in size");
    std::vector<std::string> inputs, exprs;
    for (auto& d : input_signature) inputs.push_back(d.get_name());
    for (auto& g : graphs) exprs.push_back(g->get_kernel());
    kind_ = kahan_summation ? MF_KERNEL_REDUCE : MF_KERNEL_STORE;
    nevents_ = nevents;
    nout_ = uint32_t(graphs.size());
    if (kahan_summation) kahan_.assign(nout_, evalT(0));
    if (!ready()) {
      lower_only(name, inputs, params, exprs);
      return false;
    }
    return build(name, inputs, params, exprs, nullptr, nullptr, nullptr, 0.0);
  }

  virtual bool SubmitKernel() override {
    if (!kernel_) return fail("SubmitKernel: no kernel");
    std::vector<double> p(params_.begin(), params_.end());
    const double* pp = p.empty() ? nullptr : p.data();
    if (kind_ == MF_KERNEL_REDUCE) {
      if (!input_ || !input_->buf) return fail("SubmitKernel: no input events on the device");
      std::vector<double> sums(nout_);
      if (check(mf_kernel_reduce(kernel_, input_->buf, input_->stride, nevents_, pp, uint32_t(p.size()), sums.data())))
        return false;
      kahan_.resize(nout_);
      for (uint32_t j = 0; j < nout_; j++) kahan_[j] = evalT(sums[j]);
      return true;
    }
    if (!output_) output_ = std::make_shared<Columns>(backend_->context(), kElem);
    if (kind_ == MF_KERNEL_STORE) {
      if (!input_ || !input_->buf) return fail("SubmitKernel: no input events on the device");
      if (check(output_->ensure(nout_, nevents_))) return false;
      return !check(mf_kernel_store(kernel_, input_->buf, input_->stride, nevents_, pp, uint32_t(p.size()),
                                    output_->buf, output_->stride));
    }
    // generate: the reference's accelerator partition over opencl_max_generator_workitems threads
    uint64_t nper = 0;
    uint32_t nseeds = 0;
    const int maxw = backend_->opts_->opencl_max_generator_workitems;
    if (check(mf_generate_partition(nevents_, maxw > 0 ? uint32_t(maxw) : 0u, &nper, &nseeds))) return false;
    if (seed_rows_ < nseeds) return fail("SubmitKernel: fewer seed rows than generator threads");
    std::vector<uint32_t> compact(size_t(4) * nseeds);
    for (int k = 0; k < 4; k++)
      std::memcpy(&compact[size_t(k) * nseeds], &seeds_[size_t(k) * seed_rows_], nseeds * sizeof(uint32_t));
    if (check(output_->ensure(ndims_, nevents_))) return false;
    return !check(mf_kernel_generate(kernel_, compact.data(), nseeds, nevents_, nper, pp, uint32_t(p.size()),
                                     output_->buf, output_->stride, 10000ull * nper));
  }
  virtual bool Finish() override { return ready() && !check(mf_context_synchronize(backend_->context())); }
  virtual bool ProvidesKahan() override { return true; }

  // ---- extras ----
  const std::string& last_error() const { return error_; }
  // CUDA C generated for the last Make*Kernel call (also available without a GPU).
  const std::string& kernel_source() const { return source_; }

 private:
  bool ready() {
    if (backend_ && backend_->ok()) return true;
    return fail(std::string("no CUDA context: ") + (backend_ ? backend_->error() : "null backend"));
  }
  bool fail(const std::string& msg) {
    error_ = msg;
    if (backend_ && !backend_->cuda_opts().quiet) std::cerr << "CUDABlock: " << msg << std::endl;
    return false;
  }
  int check(int rc) {
    if (rc != MF_OK) fail(mf_last_error());
    return rc;
  }
  static std::vector<const char*> cstr(const std::vector<std::string>& v) {
    std::vector<const char*> r;
    for (auto& s : v) r.push_back(s.c_str());
    return r;
  }
  mf_kernel_desc desc(const std::string& name, const std::vector<const char*>& in, const std::vector<const char*>& pa,
                      const std::vector<const char*>& ex) const {
    mf_kernel_desc d;
    std::memset(&d, 0, sizeof d);
    d.name = name.c_str();
    d.kind = kind_;
    d.elem_type = kElem;
    d.n_inputs = uint32_t(in.size());
    d.input_names = in.data();
    d.n_params = uint32_t(pa.size());
    d.param_names = pa.data();
    d.n_outputs = uint32_t(ex.size());
    d.exprs = ex.data();
    return d;
  }
  void lower_only(const std::string& name, const std::vector<std::string>& inputs,
                  const std::vector<std::string>& params, const std::vector<std::string>& exprs) {
    auto in = cstr(inputs), pa = cstr(params), ex = cstr(exprs);
    mf_kernel_desc d = desc(name, in, pa, ex);
    size_t need = 0;
    if (mf_lower_source(&d, nullptr, 0, &need) != MF_OK) return;
    source_.assign(need, '\0');
    mf_lower_source(&d, &source_[0], need, nullptr);
    source_.resize(need ? need - 1 : 0);
    print_source();
  }
  void print_source() const {
    if (backend_ && backend_->opts_ && backend_->opts_->print_kernel)
      std::cout << std::endl << "CUDA KERNEL SOURCECODE:" << std::endl << source_ << "END KERNEL SOURCECODE" << std::endl;
  }
  bool build(const std::string& name, const std::vector<std::string>& inputs, const std::vector<std::string>& params,
             const std::vector<std::string>& exprs, const std::vector<std::string>* dims,
             const std::vector<double>* lo, const std::vector<double>* hi, double maxprob) {
    if (kernel_) mf_kernel_free(kernel_);
    kernel_ = nullptr;
    auto in = cstr(inputs), pa = cstr(params), ex = cstr(exprs);
    std::vector<const char*> gd;
    mf_kernel_desc d = desc(name, in, pa, ex);
    if (dims) {
      gd = cstr(*dims);
      d.n_gen_dims = uint32_t(gd.size());
      d.gen_dim_names = gd.data();
      d.gen_lo = lo->data();
      d.gen_hi = hi->data();
      d.maxprob = maxprob;
    }
    if (check(mf_kernel_build(backend_->context(), &d, &kernel_))) return false;
    size_t need = 0;
    mf_kernel_source(kernel_, nullptr, 0, &need);
    source_.assign(need, '\0');
    mf_kernel_source(kernel_, &source_[0], need, nullptr);
    source_.resize(need ? need - 1 : 0);
    print_source();
    return true;
  }

  CUDABackend* backend_;
  const int kElem;  // element type of the device columns and kernels
  std::shared_ptr<Columns> input_, output_;
  std::vector<kernelT> params_;
  std::vector<evalT> kahan_;
  std::vector<seedT> seeds_;
  uint64_t seed_rows_ = 0;
  mf_kernel* kernel_ = nullptr;
  int kind_ = MF_KERNEL_REDUCE;
  unsigned nevents_ = 0;
  uint32_t nout_ = 0, ndims_ = 0;
  std::string error_, source_;
};

}  // namespace morefit

#endif
