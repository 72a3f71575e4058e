// Runtime of the MoreFit CUDA backend: contexts, device buffers, NVRTC
// compilation of lowered kernels, and launches (C ABI in morefit_cuda.h).
//
// Everything here is host code on the CUDA runtime API; the kernels are the
// generated translation units of mf_lower.cpp, compiled by NVRTC to sm_103a
// cubins and loaded with cudaLibraryLoadData. No entry point aborts: errors
// become MF_ERR_* codes with a thread-local message.
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <fcntl.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <thread>
#include <vector>

#include "../../include/morefit_cuda.h"
#include "mf_internal.h"
#include "mf_lower.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

}  // namespace

int set_error(int code, const std::string& msg) { return fail(code, msg); }

namespace {

#define MF_CUDA_TRY(call)                                                                                  \
  do {                                                                                                     \
    cudaError_t e_ = (call);                                                                               \
    if (e_ != cudaSuccess) return fail(MF_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// ------------------------------------------------------------ compile cache --
struct CompiledImage {
  std::vector<char> cubin;
  int regs = -1, spill = -1;
  std::string log;
};

std::mutex g_cache_mu;
std::map<std::string, std::shared_ptr<CompiledImage>> g_cache;  // key: source

uint64_t fnv1a64(const std::string& s) {
  uint64_t h = 1469598103934665603ULL;
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ULL;
  }
  return h;
}

std::string cache_dir() {
  const char* d = std::getenv("MOREFIT_CUDA_CACHE");
  if (d && *d) return d;
  const char* x = std::getenv("XDG_CACHE_HOME");
  if (x && *x) return std::string(x) + "/morefit_gb300";
  const char* h = std::getenv("HOME");
  return std::string(h ? h : "/tmp") + "/.cache/morefit_gb300";
}

void parse_ptxas_log(const std::string& log, int& regs, int& spill, const std::string& entry = "") {
  // "Compiling entry function 'NAME'" ... "Used 40 registers" ... "N bytes spill stores"
  size_t start = 0;
  if (!entry.empty()) {
    size_t e = log.find("entry function '" + entry + "'");
    if (e != std::string::npos) start = e;
  }
  size_t p = log.find("Used ", start);
  if (p != std::string::npos) regs = std::atoi(log.c_str() + p + 5);
  size_t q = log.find(" bytes spill stores", start);
  if (q != std::string::npos) {
    size_t b = q;
    while (b > 0 && (std::isdigit((unsigned char)log[b - 1]))) b--;
    spill = std::atoi(log.c_str() + b);
  }
}

int compile_source(const std::string& src, const std::string& name, std::shared_ptr<CompiledImage>& out,
                   const std::string& entry) {
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    auto it = g_cache.find(src);
    if (it != g_cache.end()) {
      out = it->second;
      return MF_OK;
    }
  }
  auto img = std::make_shared<CompiledImage>();
  char hex[32];
  std::snprintf(hex, sizeof hex, "%016llx", (unsigned long long)fnv1a64(src));
  const std::string dir = cache_dir();
  const std::string base = dir + "/k" + hex + "_sm103a";
  bool from_disk = false;
  if (!std::getenv("MOREFIT_CUDA_NOCACHE")) {
    std::ifstream f(base + ".cubin", std::ios::binary);
    std::ifstream s(base + ".src", std::ios::binary);
    if (f && s) {
      std::string cached_src((std::istreambuf_iterator<char>(s)), std::istreambuf_iterator<char>());
      if (cached_src == src) {
        img->cubin.assign((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
        std::ifstream l(base + ".log");
        if (l) img->log.assign((std::istreambuf_iterator<char>(l)), std::istreambuf_iterator<char>());
        parse_ptxas_log(img->log, img->regs, img->spill, entry);
        from_disk = !img->cubin.empty();
      }
    }
  }
  if (!from_disk) {
    nvrtcProgram prog;
    nvrtcResult r = nvrtcCreateProgram(&prog, src.c_str(), (name + ".cu").c_str(), 0, nullptr, nullptr);
    if (r != NVRTC_SUCCESS) return fail(MF_ERR_NVRTC, std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r));
    const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "--generate-line-info",
                          "--ptxas-options=-v", "--fmad=true"};
    r = nvrtcCompileProgram(prog, int(sizeof(opts) / sizeof(opts[0])), opts);
    size_t logsz = 0;
    nvrtcGetProgramLogSize(prog, &logsz);
    std::string log(logsz, '\0');
    if (logsz) nvrtcGetProgramLog(prog, &log[0]);
    img->log = log;
    if (r != NVRTC_SUCCESS) {
      nvrtcDestroyProgram(&prog);
      return fail(MF_ERR_NVRTC, "NVRTC compile of '" + name + "' failed: " + log.substr(0, 4000));
    }
    size_t cubsz = 0;
    nvrtcGetCUBINSize(prog, &cubsz);
    img->cubin.resize(cubsz);
    nvrtcGetCUBIN(prog, img->cubin.data());
    nvrtcDestroyProgram(&prog);
    parse_ptxas_log(log, img->regs, img->spill, entry);
    if (!std::getenv("MOREFIT_CUDA_NOCACHE")) {
      std::string cmd_dir = dir;
      // best effort: create the cache directory chain
      for (size_t p = 1; p <= cmd_dir.size(); p++)
        if (p == cmd_dir.size() || cmd_dir[p] == '/') ::mkdir(cmd_dir.substr(0, p).c_str(), 0755);
      std::string tmp = base + ".tmp" + std::to_string(::getpid());
      std::ofstream(tmp + ".src", std::ios::binary) << src;
      std::ofstream(tmp + ".log", std::ios::binary) << log;
      {
        std::ofstream c(tmp + ".cubin", std::ios::binary);
        c.write(img->cubin.data(), std::streamsize(img->cubin.size()));
      }
      std::rename((tmp + ".src").c_str(), (base + ".src").c_str());
      std::rename((tmp + ".log").c_str(), (base + ".log").c_str());
      std::rename((tmp + ".cubin").c_str(), (base + ".cubin").c_str());
    }
  }
  std::lock_guard<std::mutex> lk(g_cache_mu);
  g_cache[src] = img;
  out = img;
  return MF_OK;
}

}  // namespace

// ----------------------------------------------------------------- objects --
struct ResState;  // resident evaluations of a context (the resident runtime below)

struct mf_context {
  // Owner reference plus one per live buffer and kernel: the context (stream,
  // scratch) outlives everything allocated through it, whatever order the
  // caller releases handles in.
  std::atomic<int> refs{1};
  bool destroyed = false;
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  uint64_t budget = 0;
  std::atomic<uint64_t> allocated{0};
  // scratch for the grid-level combine of REDUCE kernels
  double* partials = nullptr;
  size_t partials_cap = 0;  // doubles
  unsigned* counter = nullptr;
  unsigned* status = nullptr;       // device-visible alias of status_host
  unsigned* status_host = nullptr;  // mapped pinned host words: [0] kernel error flags, [1] sync completion
  unsigned sync_seq = 0;            // sequence number of the last synchronous evaluation
  // mapped pinned host memory the kernels write results into
  double* out_host = nullptr;
  double* out_dev = nullptr;
  size_t out_cap = 0;  // doubles
  // device staging for segment tables and parameter rows
  void* stage_dev = nullptr;
  size_t stage_cap = 0;
  // freed buffer memory kept for reuse (size -> pointer), up to cache_limit
  // bytes: a server admitting and retiring datasets does not pay a
  // cudaMalloc / cudaFree (which synchronises the device) for each
  std::multimap<uint64_t, void*> free_cache;
  uint64_t cached = 0, cache_limit = 0;
  // page-locked staging of the file loader: two chunks, each reused once
  // the copy out of it (recorded event) has completed
  void* load_stage[2] = {nullptr, nullptr};
  cudaEvent_t load_done[2] = {nullptr, nullptr};
  // batched evaluations: one slot of per-block partials per evaluation of a
  // chunk, and the chunk's grid sizes
  float2* ring = nullptr;
  size_t ring_cap = 0;  // float2
  unsigned* ring_grids = nullptr;
  size_t ring_grids_cap = 0;
  // synchronous evaluations routed through a coalescer (mf_context_set_coalescer)
  mf_coalescer* coalescer = nullptr;
  // resident evaluations (mf_context_set_resident): idle time after which the
  // resident grid exits (0: off), and their state
  uint64_t res_idle_ns = 0;
  ResState* res = nullptr;
};

// A copy of a buffer's columns in the layout a REDUCE kernel reads (folded
// columns, FP64 values pre-split into float pairs), made by the kernel's
// prep pass and kept until the buffer is written again.
struct mf_derived {
  uint64_t key = 0;  // what was derived (same key: same columns, same layout)
  uint64_t gen = 0, n = 0, stride = 0;
  void* ptr = nullptr;
  uint64_t bytes = 0;  // allocated bytes (counted in the context's budget)
};

struct mf_buffer {
  mf_context* ctx = nullptr;
  void* ptr = nullptr;
  uint64_t size = 0;
  uint64_t gen = 1;  // write generation: bumped by every write through the library
  mutable std::vector<mf_derived> derived;
  // host memory the device reads in place (mf_buffer_wrap_host): not owned;
  // `registered` when this library registered it and unregisters on free
  void* host = nullptr;
  bool registered = false;
};

// Owned copy of a kernel description (its strings and arrays), kept by
// double-float REDUCE kernels to build their native-FP64 twin on demand.
struct DescCopy {
  std::string name;
  std::vector<std::string> inputs, params, exprs, defs;
  std::vector<const char*> p_inputs, p_params, p_exprs, p_defs;
  mf_kernel_desc d{};
  explicit DescCopy(const mf_kernel_desc* s) : d(*s) {
    name = s->name ? s->name : "kernel";
    for (uint32_t i = 0; i < s->n_inputs; i++) inputs.emplace_back(s->input_names[i]);
    for (uint32_t i = 0; i < s->n_params; i++) params.emplace_back(s->param_names[i]);
    for (uint32_t i = 0; i < s->n_outputs; i++) exprs.emplace_back(s->exprs[i]);
    if (s->param_defs)
      for (uint32_t i = 0; i < s->n_params; i++) defs.emplace_back(s->param_defs[i] ? s->param_defs[i] : "");
    for (auto& x : inputs) p_inputs.push_back(x.c_str());
    for (auto& x : params) p_params.push_back(x.c_str());
    for (auto& x : exprs) p_exprs.push_back(x.c_str());
    for (auto& x : defs) p_defs.push_back(x.c_str());
    d.name = name.c_str();
    d.input_names = p_inputs.data();
    d.param_names = p_params.data();
    d.exprs = p_exprs.data();
    d.param_defs = s->param_defs ? p_defs.data() : nullptr;
    d.n_gen_dims = 0;
    d.gen_dim_names = nullptr;
    d.gen_lo = d.gen_hi = nullptr;
  }
};

struct mf_kernel {
  mf_context* ctx = nullptr;
  std::string name;
  int kind = MF_KERNEL_REDUCE;
  int elem = MF_F64;
  uint32_t n_inputs = 0, n_params = 0, n_outputs = 0, n_gen_dims = 0;
  mf::LoweredKernel lowered;
  std::shared_ptr<CompiledImage> image;
  cudaLibrary_t lib = nullptr;
  cudaKernel_t fn = nullptr;
  cudaKernel_t fn_seg = nullptr;
  cudaKernel_t fn_prep = nullptr;  // REDUCE kernels reading prepared columns
  cudaKernel_t fn_part = nullptr;     // REDUCE: per-block partials only (batched evaluations)
  cudaKernel_t fn_combine = nullptr;  // REDUCE: one block per batched evaluation
  cudaKernel_t fn_multi = nullptr;    // REDUCE: segments of many datasets in one launch
  uint64_t prep_key = 0;
  int blocks_per_sm = 1;
  int max_input = -1;
  bool holds_ref = false;  // counted in ctx->refs
  // Double-float REDUCE kernels: the description, and the native-FP64 build
  // of it that re-evaluates launches whose sums came out non-finite.
  std::unique_ptr<DescCopy> desc;
  mf_kernel* f64 = nullptr;
  uint64_t fallbacks = 0;
};

namespace mfi {
int launch_reduce(mf_kernel* k, const void* data, uint64_t stride, uint64_t n, const double* params,
                  double* partials, unsigned* counter, double* out, cudaStream_t stream, int grid_cap,
                  bool dependent = false, unsigned seq = 0);
}

// ---------------------------------------------------------------- helpers --
namespace {

void res_shutdown(mf_context* c);
void res_drop(mf_context* c);
void res_yield(mf_context* c);
void res_forget(mf_kernel* k);

void release_context(mf_context* c) {
  if (!c) return;
  if (c->refs.fetch_sub(1) != 1) return;
  cudaSetDevice(c->device);
  res_shutdown(c);
  cudaStreamSynchronize(c->stream);
  if (c->partials) cudaFree(c->partials);
  if (c->counter) cudaFree(c->counter);
  if (c->out_host) cudaFreeHost(c->out_host);
  if (c->status_host) cudaFreeHost(c->status_host);
  if (c->stage_dev) cudaFree(c->stage_dev);
  if (c->ring) cudaFree(c->ring);
  if (c->ring_grids) cudaFree(c->ring_grids);
  for (int i = 0; i < 2; i++) {
    if (c->load_stage[i]) cudaFreeHost(c->load_stage[i]);
    if (c->load_done[i]) cudaEventDestroy(c->load_done[i]);
  }
  for (auto& [sz, q] : c->free_cache) cudaFree(q);
  cudaStreamDestroy(c->stream);
  delete c;
}


size_t elem_size(int e) { return e == MF_F32 ? 4 : 8; }

// Device memory for buffers and prepared copies: a cached block of the same
// rounded size (within 1/8) when one is free, else cudaMalloc; when that
// fails, the cache is released and the allocation tried once more.
cudaError_t ctx_malloc(mf_context* c, uint64_t bytes, void** p) {
  auto it = c->free_cache.lower_bound(bytes);
  if (it != c->free_cache.end() && it->first <= bytes + bytes / 8) {
    *p = it->second;
    c->cached -= it->first;
    c->free_cache.erase(it);
    return cudaSuccess;
  }
  cudaError_t e = cudaMalloc(p, std::max<uint64_t>(bytes, 256));
  if (e == cudaErrorMemoryAllocation && !c->free_cache.empty()) {
    cudaGetLastError();
    for (auto& [sz, q] : c->free_cache) cudaFree(q);
    c->free_cache.clear();
    c->cached = 0;
    e = cudaMalloc(p, std::max<uint64_t>(bytes, 256));
  }
  return e;
}
// Returns memory of `bytes` (the size it was allocated with) for reuse; the
// caller has synchronised the context's stream.
void ctx_free(mf_context* c, void* p, uint64_t bytes) {
  if (!p) return;
  if (c->cached + bytes <= c->cache_limit) {
    c->free_cache.emplace(bytes, p);
    c->cached += bytes;
  } else {
    cudaFree(p);
  }
}

// Reads (and clears) the kernels' error word after the stream has drained.
int check_status(mf_context* c) {
  const unsigned st = *c->status_host;
  if (!st) return MF_OK;
  *c->status_host = 0u;
  cudaMemsetAsync(c->counter, 0, sizeof(unsigned), c->stream);  // a block that gave up may have left it set
  cudaStreamSynchronize(c->stream);
  return fail(MF_ERR_TIMEOUT, "a kernel gave up waiting for its input tiles (status " + std::to_string(st) + ")");
}

// Waits for the synchronous evaluation `seq`: its combining block stores
// seq in the mapped word status[1] once the sums are visible to the host.
// The host spins on that word (a stream synchronize costs about 1.6 us more
// per call); past kSyncSpinUs, or if the launch failed, it falls back to a
// stream synchronize, which also reports any asynchronous error.
int wait_sync_word(mf_context* c, unsigned seq) {
  constexpr auto kSyncSpinUs = std::chrono::microseconds(500);
  const auto t0 = std::chrono::steady_clock::now();
  unsigned spins = 0;
  while (__atomic_load_n(c->status_host + 1, __ATOMIC_ACQUIRE) != seq) {
    if ((++spins & 255u) == 0 && std::chrono::steady_clock::now() - t0 > kSyncSpinUs) {
      MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
      break;
    }
  }
  return MF_OK;
}

int ensure_scratch(mf_context* c, size_t partial_doubles, size_t out_doubles) {
  if (partial_doubles > c->partials_cap) {
    if (c->partials) cudaFree(c->partials);
    c->partials = nullptr;
    size_t cap = std::max<size_t>(partial_doubles, 1 << 16);
    MF_CUDA_TRY(cudaMalloc(&c->partials, cap * sizeof(double)));
    c->partials_cap = cap;
  }
  if (out_doubles > c->out_cap) {
    if (c->out_host) cudaFreeHost(c->out_host);
    c->out_host = nullptr;
    size_t cap = std::max<size_t>(out_doubles, 4096);
    MF_CUDA_TRY(cudaHostAlloc(reinterpret_cast<void**>(&c->out_host), cap * sizeof(double), cudaHostAllocMapped));
    MF_CUDA_TRY(cudaHostGetDevicePointer(reinterpret_cast<void**>(&c->out_dev), c->out_host, 0));
    c->out_cap = cap;
  }
  return MF_OK;
}

int ensure_stage(mf_context* c, size_t bytes) {
  if (bytes > c->stage_cap) {
    if (c->stage_dev) cudaFree(c->stage_dev);
    c->stage_dev = nullptr;
    size_t cap = std::max<size_t>(bytes, 1 << 20);
    MF_CUDA_TRY(cudaMalloc(&c->stage_dev, cap));
    c->stage_cap = cap;
  }
  return MF_OK;
}

int check_layout(const mf_kernel* k, const mf_buffer* in, uint64_t stride, uint64_t n) {
  if (!in || !in->ptr) return fail(MF_ERR_INVALID, "input buffer is null");
  if (stride < n) return fail(MF_ERR_INVALID, "column stride smaller than the number of events");
  if (k->kind == MF_KERNEL_REDUCE && (stride % uint64_t(std::max(1, k->lowered.vec)) != 0))
    return fail(MF_ERR_INVALID, "column stride is not a multiple of the kernel's vector width");
  if ((reinterpret_cast<uintptr_t>(in->ptr) & 15u) != 0) return fail(MF_ERR_INVALID, "input buffer not 16-byte aligned");
  const uint64_t need = uint64_t(k->max_input + 1) * stride * elem_size(k->elem);
  if (k->max_input >= 0 && need > in->size)
    return fail(MF_ERR_INVALID, "input buffer smaller than columns x stride (" + std::to_string(need) + " > " +
                                    std::to_string(in->size) + " bytes)");
  return MF_OK;
}

uint64_t fnv1a(const void* p, size_t n, uint64_t h = 0xcbf29ce484222325ULL) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; i++) h = (h ^ b[i]) * 0x100000001b3ULL;
  return h;
}

uint64_t prep_key(const mf_kernel* k) {
  const auto& lk = k->lowered;
  uint64_t h = fnv1a(&lk.prep, sizeof lk.prep);
  h = fnv1a(&k->elem, sizeof k->elem, h);
  for (const auto& col : lk.prep_cols) {
    const uint64_t nt = col.size();
    h = fnv1a(&nt, sizeof nt, h);
    for (const auto& [src, c] : col) {
      h = fnv1a(&src, sizeof src, h);
      h = fnv1a(&c, sizeof c, h);
    }
  }
  return h;
}

// The device columns kernel `k` reads for input buffer `in`: the buffer
// itself, or its prepared copy, (re)made on the context's stream when the
// buffer was written since (or the column stride changed). The copy covers
// all `stride` rows of the columns, so evaluations of any event count or
// segment of the buffer share it (event loops never accumulate rows at or
// beyond their n).
int prepare_input(const mf_kernel* k, const mf_buffer* in, uint64_t stride, const void** data) {
  if (!k->lowered.prep) {
    *data = in->ptr;
    return MF_OK;
  }
  mf_context* c = k->ctx;
  mf_derived* d = nullptr;
  for (auto& x : in->derived)
    if (x.key == k->prep_key) d = &x;
  if (d && d->gen == in->gen && d->stride == stride) {
    *data = d->ptr;
    return MF_OK;
  }
  const uint64_t need = (uint64_t(k->lowered.prep_cols.size()) * stride * k->lowered.prep_elem_bytes() + 255) &
                        ~uint64_t(255);
  if (!d || d->bytes < need) {
    const uint64_t old = d ? d->bytes : 0;
    if (c->budget && c->allocated.load() - old + need > c->budget)
      return fail(MF_ERR_BUDGET, "the prepared copy of an input (" + std::to_string(need) +
                                     " bytes) exceeds the HBM budget");
    if (d && d->ptr) {
      MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
      ctx_free(c, d->ptr, d->bytes);
      c->allocated -= d->bytes;
      d->ptr = nullptr;
      d->bytes = 0;
    }
    if (!d) {
      in->derived.push_back(mf_derived{});
      d = &in->derived.back();
      d->key = k->prep_key;
    }
    MF_CUDA_TRY(ctx_malloc(c, need, &d->ptr));
    d->bytes = need;
    c->allocated += need;
  }
  const uint64_t blocks = (stride + 255) / 256;
  const int grid = int(std::max<uint64_t>(1, std::min<uint64_t>(blocks, uint64_t(c->num_sms) * 16)));
  const void* src = in->ptr;
  void* dst = d->ptr;
  uint64_t rows = stride;
  void* args[] = {const_cast<void**>(&src), &stride, &rows, &dst};
  res_yield(c);
  MF_CUDA_TRY(cudaLaunchKernel(reinterpret_cast<const void*>(k->fn_prep), dim3(grid), dim3(256), args, 0, c->stream));
  d->gen = in->gen;
  d->n = stride;
  d->stride = stride;
  *data = d->ptr;
  return MF_OK;
}

void free_derived(const mf_buffer* b) {
  for (auto& d : b->derived)
    if (d.ptr) {
      ctx_free(b->ctx, d.ptr, d.bytes);
      b->ctx->allocated -= d.bytes;
    }
  b->derived.clear();
}

}  // namespace

// ------------------------------------------------------------------ C ABI --
extern "C" {

const char* mf_last_error(void) { return g_last_error.c_str(); }

const char* mf_version(void) { return "morefit_gb300 0.1 (sm_103a, NVRTC)"; }

int mf_device_count(int* count) {
  if (!count) return fail(MF_ERR_INVALID, "count is null");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  *count = n;
  return MF_OK;
}

int mf_device_properties(int device, char* name, size_t len, int* sm_count, int* cc_major, int* cc_minor) {
  int n = 0;
  mf_device_count(&n);
  if (n == 0) return fail(MF_ERR_NO_DEVICE, "no CUDA device");
  if (device < 0 || device >= n) return fail(MF_ERR_INVALID, "device index out of range");
  cudaDeviceProp p;
  MF_CUDA_TRY(cudaGetDeviceProperties(&p, device));
  if (name && len) {
    std::strncpy(name, p.name, len - 1);
    name[len - 1] = 0;
  }
  if (sm_count) *sm_count = p.multiProcessorCount;
  if (cc_major) *cc_major = p.major;
  if (cc_minor) *cc_minor = p.minor;
  return MF_OK;
}

int mf_context_create(int device, uint64_t hbm_budget_bytes, mf_context** out) {
  if (!out) return fail(MF_ERR_INVALID, "out is null");
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(MF_ERR_NO_DEVICE, "no CUDA device visible");
  }
  if (device < 0 || device >= n) return fail(MF_ERR_INVALID, "device index out of range");
  MF_CUDA_TRY(cudaSetDevice(device));
  cudaDeviceProp prop;
  MF_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10 || prop.minor != 3)
    return fail(MF_ERR_NO_DEVICE, std::string("device is sm_") + std::to_string(prop.major) +
                                      std::to_string(prop.minor) + ", this build targets sm_103a (GB300)");
  auto c = std::make_unique<mf_context>();
  c->device = device;
  c->num_sms = prop.multiProcessorCount;
  c->budget = hbm_budget_bytes;
  c->cache_limit = hbm_budget_bytes ? hbm_budget_bytes / 4 : (uint64_t(8) << 30);
  MF_CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  MF_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&c->counter), sizeof(unsigned)));
  MF_CUDA_TRY(cudaMemset(c->counter, 0, sizeof(unsigned)));
  MF_CUDA_TRY(cudaHostAlloc(reinterpret_cast<void**>(&c->status_host), 64, cudaHostAllocMapped));
  MF_CUDA_TRY(cudaHostGetDevicePointer(reinterpret_cast<void**>(&c->status), c->status_host, 0));
  // all words: [1] is the completion word the first synchronous call waits
  // for, and page-locked memory comes back from earlier allocations unzeroed
  std::memset(c->status_host, 0, 64);
  int rc = ensure_scratch(c.get(), size_t(c->num_sms) * 8 * 64, 4096);
  if (rc) return rc;
  *out = c.release();
  return MF_OK;
}

int mf_context_destroy(mf_context* c) {
  if (!c) return MF_OK;
  if (c->destroyed) return fail(MF_ERR_INVALID, "context destroyed twice");
  c->destroyed = true;
  if (c->res) {
    cudaSetDevice(c->device);
    res_drop(c);  // the resident grid leaves now, not when the last kernel is freed
    c->res_idle_ns = 0;
  }
  release_context(c);
  return MF_OK;
}

int mf_context_allocated(const mf_context* c, uint64_t* bytes) {
  if (!c || !bytes) return fail(MF_ERR_INVALID, "null argument");
  *bytes = c->allocated.load();
  return MF_OK;
}

int mf_context_synchronize(mf_context* c) {
  if (!c) return fail(MF_ERR_INVALID, "context is null");
  MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return check_status(c);
}

int mf_buffer_alloc(mf_context* c, uint64_t nbytes, mf_buffer** out) {
  if (!c || !out) return fail(MF_ERR_INVALID, "null argument");
  *out = nullptr;
  const uint64_t rounded = (nbytes + 255) & ~uint64_t(255);
  if (c->budget && c->allocated.load() + rounded > c->budget)
    return fail(MF_ERR_BUDGET, "allocation of " + std::to_string(rounded) + " bytes exceeds the HBM budget (" +
                                   std::to_string(c->allocated.load()) + " of " + std::to_string(c->budget) +
                                   " bytes in use)");
  MF_CUDA_TRY(cudaSetDevice(c->device));
  auto b = std::make_unique<mf_buffer>();
  b->ctx = c;
  b->size = nbytes;
  MF_CUDA_TRY(ctx_malloc(c, std::max<uint64_t>(rounded, 256), &b->ptr));
  c->allocated += rounded;
  c->refs++;
  *out = b.release();
  return MF_OK;
}

int mf_buffer_free(mf_buffer* b) {
  if (!b) return MF_OK;
  mf_context* c = b->ctx;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_derived(b);
  if (b->host) {
    if (b->registered) cudaHostUnregister(b->host);
  } else {
    ctx_free(c, b->ptr, std::max<uint64_t>((b->size + 255) & ~uint64_t(255), 256));
    c->allocated -= (b->size + 255) & ~uint64_t(255);
  }
  delete b;
  release_context(c);
  return MF_OK;
}

int mf_buffer_wrap_host(mf_context* c, void* host, uint64_t nbytes, mf_buffer** out) {
  if (!c || !host || !out) return fail(MF_ERR_INVALID, "null argument");
  *out = nullptr;
  MF_CUDA_TRY(cudaSetDevice(c->device));
  auto b = std::make_unique<mf_buffer>();
  b->ctx = c;
  b->size = nbytes;
  b->host = host;
  void* d = nullptr;
  if (cudaHostGetDevicePointer(&d, host, 0) != cudaSuccess) {
    cudaGetLastError();  // not page-locked yet: register it (mapped) for this buffer's lifetime
    MF_CUDA_TRY(cudaHostRegister(host, nbytes, cudaHostRegisterMapped));
    b->registered = true;
    const cudaError_t e = cudaHostGetDevicePointer(&d, host, 0);
    if (e != cudaSuccess) {
      cudaHostUnregister(host);
      return fail(MF_ERR_CUDA, std::string("cudaHostGetDevicePointer: ") + cudaGetErrorString(e));
    }
  }
  b->ptr = d;
  c->refs++;
  *out = b.release();
  return MF_OK;
}

uint64_t mf_buffer_size(const mf_buffer* b) { return b ? b->size : 0; }

void* mf_buffer_device_ptr(const mf_buffer* b) { return b ? b->ptr : nullptr; }

int mf_buffer_mark_modified(mf_buffer* b) {
  if (!b) return fail(MF_ERR_INVALID, "null buffer");
  b->gen++;
  return MF_OK;
}

int mf_buffer_h2d(mf_buffer* b, uint64_t off, const void* src, uint64_t nbytes) {
  if (!b || (!src && nbytes)) return fail(MF_ERR_INVALID, "null argument");
  if (off + nbytes > b->size) return fail(MF_ERR_INVALID, "copy beyond the end of the buffer");
  MF_CUDA_TRY(cudaSetDevice(b->ctx->device));
  b->gen++;
  MF_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(b->ptr) + off, src, nbytes, cudaMemcpyHostToDevice, b->ctx->stream));
  MF_CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
  return MF_OK;
}

int mf_buffer_d2h(const mf_buffer* b, uint64_t off, void* dst, uint64_t nbytes) {
  if (!b || (!dst && nbytes)) return fail(MF_ERR_INVALID, "null argument");
  if (off + nbytes > b->size) return fail(MF_ERR_INVALID, "copy beyond the end of the buffer");
  MF_CUDA_TRY(cudaSetDevice(b->ctx->device));
  MF_CUDA_TRY(cudaMemcpyAsync(dst, static_cast<const char*>(b->ptr) + off, nbytes, cudaMemcpyDeviceToHost,
                              b->ctx->stream));
  MF_CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
  return MF_OK;
}

int mf_buffer_memset(mf_buffer* b, int value) {
  if (!b) return fail(MF_ERR_INVALID, "null buffer");
  MF_CUDA_TRY(cudaSetDevice(b->ctx->device));
  b->gen++;
  MF_CUDA_TRY(cudaMemsetAsync(b->ptr, value, b->size, b->ctx->stream));
  MF_CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
  return MF_OK;
}

uint64_t mf_column_stride(uint64_t n) {
  const uint64_t a = MF_COLUMN_ALIGN;
  return std::max<uint64_t>(a, (n + a - 1) / a * a);
}

static int events_copy(bool up, mf_buffer* b, int elem, void* host, uint32_t ncols, uint64_t n, uint64_t hs,
                       uint64_t ds, bool sync = true) {
  if (!b || (!host && n && ncols)) return fail(MF_ERR_INVALID, "null argument");
  if (elem != MF_F64 && elem != MF_F32) return fail(MF_ERR_INVALID, "element type must be MF_F64 or MF_F32");
  const size_t es = elem_size(elem);
  if (hs < n || ds < n) return fail(MF_ERR_INVALID, "stride smaller than the number of events");
  if (uint64_t(ncols) * ds * es > b->size) return fail(MF_ERR_INVALID, "buffer smaller than ncols x stride");
  if (ncols == 0) return MF_OK;
  MF_CUDA_TRY(cudaSetDevice(b->ctx->device));
  if (up) {
    b->gen++;
    if (n && hs == ds)  // columns contiguous on both sides: one linear copy
      MF_CUDA_TRY(cudaMemcpyAsync(b->ptr, host, uint64_t(ncols) * ds * es, cudaMemcpyHostToDevice, b->ctx->stream));
    else if (n)
      MF_CUDA_TRY(cudaMemcpy2DAsync(b->ptr, ds * es, host, hs * es, n * es, ncols, cudaMemcpyHostToDevice,
                                    b->ctx->stream));
    if (ds > n)
      MF_CUDA_TRY(cudaMemset2DAsync(static_cast<char*>(b->ptr) + n * es, ds * es, 0, (ds - n) * es, ncols,
                                    b->ctx->stream));
  } else if (n && hs == ds) {
    MF_CUDA_TRY(cudaMemcpyAsync(host, b->ptr, uint64_t(ncols) * ds * es, cudaMemcpyDeviceToHost, b->ctx->stream));
  } else if (n) {
    MF_CUDA_TRY(cudaMemcpy2DAsync(host, hs * es, b->ptr, ds * es, n * es, ncols, cudaMemcpyDeviceToHost,
                                  b->ctx->stream));
  }
  if (sync) MF_CUDA_TRY(cudaStreamSynchronize(b->ctx->stream));
  return MF_OK;
}

int mf_events_upload(mf_buffer* b, int elem, const void* host, uint32_t ncols, uint64_t n, uint64_t hs, uint64_t ds) {
  return events_copy(true, b, elem, const_cast<void*>(host), ncols, n, hs, ds);
}

int mf_events_download(const mf_buffer* b, int elem, void* host, uint32_t ncols, uint64_t n, uint64_t hs,
                       uint64_t ds) {
  return events_copy(false, const_cast<mf_buffer*>(b), elem, host, ncols, n, hs, ds);
}

int mf_events_upload_async(mf_buffer* b, int elem, const void* host, uint32_t ncols, uint64_t n, uint64_t hs,
                           uint64_t ds) {
  return events_copy(true, b, elem, const_cast<void*>(host), ncols, n, hs, ds, false);
}

int mf_buffer_d2h_async(const mf_buffer* b, uint64_t off, void* dst, uint64_t nbytes) {
  if (!b || (!dst && nbytes)) return fail(MF_ERR_INVALID, "null argument");
  if (off + nbytes > b->size) return fail(MF_ERR_INVALID, "copy beyond the end of the buffer");
  MF_CUDA_TRY(cudaSetDevice(b->ctx->device));
  MF_CUDA_TRY(cudaMemcpyAsync(dst, static_cast<const char*>(b->ptr) + off, nbytes, cudaMemcpyDeviceToHost,
                              b->ctx->stream));
  return MF_OK;
}

int mf_events_upload_f64_as(mf_buffer* b, int elem, const double* host, uint32_t ncols, uint64_t n, uint64_t hs,
                            uint64_t ds) {
  if (elem == MF_F64) return mf_events_upload(b, elem, host, ncols, n, hs, ds);
  if (elem != MF_F32) return fail(MF_ERR_INVALID, "element type must be MF_F64 or MF_F32");
  std::vector<float> tmp(size_t(ncols) * n);
  for (uint32_t c = 0; c < ncols; c++)
    for (uint64_t i = 0; i < n; i++) tmp[size_t(c) * n + i] = float(host[c * hs + i]);
  return mf_events_upload(b, MF_F32, tmp.data(), ncols, n, n, ds);
}

// Reads `bytes` at `off` of fd, retrying short reads; false at end of file.
static bool read_fully(int fd, void* dst, uint64_t bytes, uint64_t off) {
  char* p = static_cast<char*>(dst);
  while (bytes) {
    const ssize_t r = pread(fd, p, size_t(std::min<uint64_t>(bytes, uint64_t(1) << 30)), off_t(off));
    if (r <= 0) return false;
    p += r;
    off += uint64_t(r);
    bytes -= uint64_t(r);
  }
  return true;
}

int mf_events_load_file(mf_buffer* b, int dev_elem, uint64_t dev_stride, const char* path, uint64_t offset,
                        int file_elem, uint64_t file_stride, uint32_t ncols, const uint32_t* cols, uint64_t n) {
  if (!b || !path || (ncols && !cols)) return fail(MF_ERR_INVALID, "null argument");
  if ((dev_elem != MF_F64 && dev_elem != MF_F32) || (file_elem != MF_F64 && file_elem != MF_F32))
    return fail(MF_ERR_INVALID, "element types must be MF_F64 or MF_F32");
  if (n > file_stride) return fail(MF_ERR_INVALID, "more events requested than a file column holds");
  if (dev_stride < n) return fail(MF_ERR_INVALID, "device column stride smaller than the number of events");
  const uint64_t fes = elem_size(file_elem), des = elem_size(dev_elem);
  if (uint64_t(ncols) * dev_stride * des > b->size)
    return fail(MF_ERR_INVALID, "buffer smaller than ncols x dev_stride elements");
  mf_context* c = b->ctx;
  MF_CUDA_TRY(cudaSetDevice(c->device));
  constexpr uint64_t kChunk = uint64_t(8) << 20;  // bytes per staging chunk
  for (int i = 0; i < 2; i++) {
    if (!c->load_stage[i]) MF_CUDA_TRY(cudaHostAlloc(&c->load_stage[i], kChunk, cudaHostAllocDefault));
    if (!c->load_done[i]) MF_CUDA_TRY(cudaEventCreateWithFlags(&c->load_done[i], cudaEventDisableTiming));
  }
  const int fd = open(path, O_RDONLY);
  if (fd < 0) return fail(MF_ERR_INVALID, std::string("cannot open ") + path);
  const uint64_t rows = kChunk / std::max(fes, des);
  std::vector<unsigned char> conv(fes != des ? size_t(rows * fes) : 0);
  char* dev = static_cast<char*>(b->ptr);
  bool recorded[2] = {false, false};
  int slot = 0, rc = MF_OK;
  b->gen++;
  for (uint32_t j = 0; j < ncols && rc == MF_OK; j++) {
    for (uint64_t r0 = 0; r0 < n && rc == MF_OK; r0 += rows) {
      const uint64_t m = std::min(rows, n - r0);
      // the staging chunk is free again once its previous copy has completed
      if (recorded[slot] && cudaEventSynchronize(c->load_done[slot]) != cudaSuccess) {
        rc = fail(MF_ERR_CUDA, "waiting for a staging copy failed");
        break;
      }
      void* st = c->load_stage[slot];
      const uint64_t foff = offset + (uint64_t(cols[j]) * file_stride + r0) * fes;
      if (!read_fully(fd, fes == des ? st : conv.data(), m * fes, foff)) {
        rc = fail(MF_ERR_INVALID, std::string("file too short: ") + path);
        break;
      }
      if (fes != des) {
        if (file_elem == MF_F64) {
          const double* s = reinterpret_cast<const double*>(conv.data());
          float* d = static_cast<float*>(st);
          for (uint64_t i = 0; i < m; i++) d[i] = float(s[i]);
        } else {
          const float* s = reinterpret_cast<const float*>(conv.data());
          double* d = static_cast<double*>(st);
          for (uint64_t i = 0; i < m; i++) d[i] = double(s[i]);
        }
      }
      if (cudaMemcpyAsync(dev + (uint64_t(j) * dev_stride + r0) * des, st, m * des, cudaMemcpyHostToDevice,
                          c->stream) != cudaSuccess ||
          cudaEventRecord(c->load_done[slot], c->stream) != cudaSuccess) {
        rc = fail(MF_ERR_CUDA, "staging copy failed");
        break;
      }
      recorded[slot] = true;
      slot ^= 1;
    }
    if (rc == MF_OK && dev_stride > n &&
        cudaMemsetAsync(dev + (uint64_t(j) * dev_stride + n) * des, 0, (dev_stride - n) * des, c->stream) !=
            cudaSuccess)
      rc = fail(MF_ERR_CUDA, "padding fill failed");
  }
  close(fd);
  MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return rc;
}

static int lower_desc(const mf_kernel_desc* d, mf::LoweredKernel& lk);

int mf_kernel_build(mf_context* c, const mf_kernel_desc* d, mf_kernel** out) {
  if (!c || !d || !out) return fail(MF_ERR_INVALID, "null argument");
  *out = nullptr;
  auto k = std::make_unique<mf_kernel>();
  k->ctx = c;
  k->name = d->name ? d->name : "kernel";
  k->kind = d->kind;
  k->elem = d->elem_type;
  k->n_inputs = d->n_inputs;
  k->n_params = d->n_params;
  k->n_outputs = d->n_outputs;
  k->n_gen_dims = d->kind == MF_KERNEL_GENERATE ? d->n_gen_dims : 0;
  int lrc = lower_desc(d, k->lowered);
  if (lrc) return lrc;
  for (int i : k->lowered.source_inputs) k->max_input = std::max(k->max_input, i);
  int rc = compile_source(k->lowered.source, k->name, k->image, k->lowered.entry);
  if (rc) return rc;
  MF_CUDA_TRY(cudaSetDevice(c->device));
  MF_CUDA_TRY(cudaLibraryLoadData(&k->lib, k->image->cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
  MF_CUDA_TRY(cudaLibraryGetKernel(&k->fn, k->lib, k->lowered.entry.c_str()));
  if (d->kind == MF_KERNEL_REDUCE || d->kind == MF_KERNEL_GENERATE)
    MF_CUDA_TRY(cudaLibraryGetKernel(&k->fn_seg, k->lib, (k->lowered.entry + "_segments").c_str()));
  if (d->kind == MF_KERNEL_REDUCE) {
    MF_CUDA_TRY(cudaLibraryGetKernel(&k->fn_part, k->lib, (k->lowered.entry + "_part").c_str()));
    MF_CUDA_TRY(cudaLibraryGetKernel(&k->fn_combine, k->lib, (k->lowered.entry + "_combine").c_str()));
    MF_CUDA_TRY(cudaLibraryGetKernel(&k->fn_multi, k->lib, (k->lowered.entry + "_multi").c_str()));
  }
  if (k->lowered.prep) {
    MF_CUDA_TRY(cudaLibraryGetKernel(&k->fn_prep, k->lib, (k->lowered.entry + "_prep").c_str()));
    k->prep_key = prep_key(k.get());
  }
  if (k->lowered.smem_bytes > 48 * 1024) {
    MF_CUDA_TRY(cudaFuncSetAttribute(reinterpret_cast<const void*>(k->fn), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(k->lowered.smem_bytes)));
    if (k->fn_part)
      MF_CUDA_TRY(cudaFuncSetAttribute(reinterpret_cast<const void*>(k->fn_part),
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(k->lowered.smem_bytes)));
  }
  int nb = 0;
  MF_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, reinterpret_cast<const void*>(k->fn),
                                                            k->lowered.block, k->lowered.smem_bytes));
  if (nb == 0)
    return fail(MF_ERR_UNSUPPORTED, "kernel '" + k->name + "' does not fit on an SM (" +
                                        std::to_string(k->lowered.smem_bytes) + " B shared memory)");
  k->blocks_per_sm = std::max(1, nb);
  const bool dw = d->kind == MF_KERNEL_REDUCE && d->elem_type == MF_F64 &&
                  !(d->flags & (MF_FLAG_NATIVE_F64 | MF_FLAG_F32_ARITH));
  // Double-float kernels of many outputs (Hessians) are issue-bound, and one
  // evaluation's grid runs them fastest at about eight warps per SM: the
  // P-wave Hessian (36 outputs, 1M events, batched) takes 25.4 us per
  // evaluation with one block of 256 threads per SM against 27.2 us with two.
  if (dw && d->n_outputs > 16)
    k->blocks_per_sm = std::min(k->blocks_per_sm, std::max(1, 256 / int(k->lowered.block)));
  if (dw) k->desc = std::make_unique<DescCopy>(d);
  c->refs++;
  k->holds_ref = true;
  *out = k.release();
  return MF_OK;
}

static int lower_desc(const mf_kernel_desc* d, mf::LoweredKernel& lk) {
  if (!d) return fail(MF_ERR_INVALID, "null descriptor");
  if (d->elem_type != MF_F64 && d->elem_type != MF_F32) return fail(MF_ERR_INVALID, "bad element type");
  if (d->kind != MF_KERNEL_REDUCE && d->kind != MF_KERNEL_STORE && d->kind != MF_KERNEL_GENERATE)
    return fail(MF_ERR_INVALID, "bad kernel kind");
  if (d->n_outputs == 0 || d->n_outputs > MF_MAX_OUTPUTS || !d->exprs)
    return fail(MF_ERR_INVALID, "bad number of outputs");
  if (d->n_params > MF_MAX_PARAMS) return fail(MF_ERR_INVALID, "too many parameters");
  auto names = [](uint32_t n, const char* const* p) {
    std::vector<std::string> v;
    for (uint32_t i = 0; i < n; i++) v.push_back(p && p[i] ? p[i] : "");
    return v;
  };
  mf::GenerateSpec gs;
  if (d->kind == MF_KERNEL_GENERATE) {
    if (d->n_outputs != 1 || d->n_gen_dims == 0 || !d->gen_lo || !d->gen_hi)
      return fail(MF_ERR_INVALID, "generate kernel needs one density expression and its dimensions");
    gs.dims = names(d->n_gen_dims, d->gen_dim_names);
    gs.lo.assign(d->gen_lo, d->gen_lo + d->n_gen_dims);
    gs.hi.assign(d->gen_hi, d->gen_hi + d->n_gen_dims);
    gs.maxprob = d->maxprob;
  }
  std::vector<std::string> defs;
  if (d->param_defs)
    for (uint32_t i = 0; i < d->n_params; i++) defs.push_back(d->param_defs[i] ? d->param_defs[i] : "");
  try {
    lk = mf::lower(d->name ? d->name : "kernel",
                   d->kind == MF_KERNEL_REDUCE  ? mf::Kind::Reduce
                   : d->kind == MF_KERNEL_STORE ? mf::Kind::Store
                                                : mf::Kind::Generate,
                   d->elem_type == MF_F32 ? mf::Elem::F32 : mf::Elem::F64, names(d->n_inputs, d->input_names),
                   names(d->n_params, d->param_names), names(d->n_outputs, d->exprs),
                   d->kind == MF_KERNEL_GENERATE ? &gs : nullptr, (d->flags & MF_FLAG_NATIVE_F64) != 0, int(d->vec),
                   int(d->block), d->elem_type == MF_F64 && (d->flags & MF_FLAG_F32_ARITH) != 0,
                   (d->flags & MF_FLAG_BULK_PIPELINE) == 0, int(d->stages), defs);
  } catch (const std::exception& e) {
    return fail(MF_ERR_PARSE, e.what());
  }
  return MF_OK;
}

int mf_lower_source(const mf_kernel_desc* d, char* buf, size_t len, size_t* needed) {
  mf::LoweredKernel lk;
  int rc = lower_desc(d, lk);
  if (rc) return rc;
  if (needed) *needed = lk.source.size() + 1;
  if (buf && len) {
    size_t n = std::min(len - 1, lk.source.size());
    std::memcpy(buf, lk.source.data(), n);
    buf[n] = '\0';
  }
  return MF_OK;
}

int mf_eval_expressions(uint32_t n_names, const char* const* names, const double* values, uint32_t n_exprs,
                        const char* const* exprs, double* out) {
  if ((n_names && (!names || !values)) || (n_exprs && (!exprs || !out))) return fail(MF_ERR_INVALID, "null argument");
  std::vector<std::string> nm;
  for (uint32_t i = 0; i < n_names; i++) nm.push_back(names[i] ? names[i] : "");
  std::vector<double> vals(values, values + n_names);
  try {
    mf::Dag dag({}, nm);
    for (uint32_t i = 0; i < n_exprs; i++) out[i] = dag.eval(dag.parse(exprs[i] ? exprs[i] : ""), {}, vals);
  } catch (const std::exception& e) {
    return fail(MF_ERR_PARSE, e.what());
  }
  return MF_OK;
}

int mf_eval_expressions_batch(uint32_t n_names, const char* const* names, uint32_t n_rows, const double* values,
                              uint32_t n_exprs, const char* const* exprs, double* out) {
  if ((n_names && !names) || (n_rows && n_names && !values) || (n_exprs && (!exprs || (n_rows && !out))))
    return fail(MF_ERR_INVALID, "null argument");
  std::vector<std::string> nm;
  for (uint32_t i = 0; i < n_names; i++) nm.push_back(names[i] ? names[i] : "");
  try {
    mf::Dag dag({}, nm);
    std::vector<int> roots;
    for (uint32_t i = 0; i < n_exprs; i++) roots.push_back(dag.parse(exprs[i] ? exprs[i] : ""));
    std::vector<double> row(n_names);
    for (uint32_t r = 0; r < n_rows; r++) {
      std::copy(values + size_t(r) * n_names, values + size_t(r + 1) * n_names, row.begin());
      for (uint32_t i = 0; i < n_exprs; i++) out[size_t(r) * n_exprs + i] = dag.eval(roots[i], {}, row);
    }
  } catch (const std::exception& e) {
    return fail(MF_ERR_PARSE, e.what());
  }
  return MF_OK;
}

}  // extern "C"

struct mf_expr_set {
  mf::Dag dag;
  std::vector<int> roots;
  uint32_t n_names = 0;
  mf_expr_set(const std::vector<std::string>& names) : dag({}, names), n_names(uint32_t(names.size())) {}
};

namespace {
// mf_spd_solve_batch for orders up to kSpdLaneOrder: kSpdLanes matrices in
// lockstep, the lane index innermost, so that the factorisations' dependent
// multiply-add chains of different matrices overlap (and vectorise). Lanes
// beyond nb factor the identity; a lane that meets a non-positive pivot
// continues on 1.0 and is reported in ok[] (its outputs are not written).
constexpr uint32_t kSpdLanes = 8, kSpdLaneOrder = 16;
void spd_lanes(uint32_t nb, uint32_t p, const double* h, const double* g, double* x, double* dinv,
               unsigned char* ok) {
  constexpr uint32_t B = kSpdLanes;
  double lf[kSpdLaneOrder][kSpdLaneOrder][B], rd[kSpdLaneOrder][B], y[kSpdLaneOrder][B], v[B];
  bool pd[B];
  for (uint32_t b = 0; b < B; b++) pd[b] = true;
  auto elem = [&](uint32_t b, uint32_t i, uint32_t j) {
    return b < nb ? h[(size_t(b) * p + i) * p + j] : (i == j ? 1.0 : 0.0);
  };
  for (uint32_t i = 0; i < p; i++) {
    for (uint32_t j = 0; j < i; j++) {
      for (uint32_t b = 0; b < B; b++) v[b] = elem(b, i, j);
      for (uint32_t k = 0; k < j; k++)
        for (uint32_t b = 0; b < B; b++) v[b] -= lf[i][k][b] * lf[j][k][b];
      for (uint32_t b = 0; b < B; b++) lf[i][j][b] = v[b] * rd[j][b];
    }
    for (uint32_t b = 0; b < B; b++) v[b] = elem(b, i, i);
    for (uint32_t k = 0; k < i; k++)
      for (uint32_t b = 0; b < B; b++) v[b] -= lf[i][k][b] * lf[i][k][b];
    for (uint32_t b = 0; b < B; b++) {
      if (!(v[b] > 0.0)) {
        pd[b] = false;
        v[b] = 1.0;
      }
      lf[i][i][b] = std::sqrt(v[b]);
      rd[i][b] = 1.0 / lf[i][i][b];
    }
  }
  for (uint32_t b = 0; b < nb; b++) ok[b] = pd[b] ? 1 : 0;
  if (g) {
    double xs[kSpdLaneOrder][B];
    for (uint32_t i = 0; i < p; i++) {
      for (uint32_t b = 0; b < B; b++) v[b] = b < nb ? g[size_t(b) * p + i] : 0.0;
      for (uint32_t k = 0; k < i; k++)
        for (uint32_t b = 0; b < B; b++) v[b] -= lf[i][k][b] * y[k][b];
      for (uint32_t b = 0; b < B; b++) y[i][b] = v[b] * rd[i][b];
    }
    for (uint32_t i = p; i-- > 0;) {
      for (uint32_t b = 0; b < B; b++) v[b] = y[i][b];
      for (uint32_t k = i + 1; k < p; k++)
        for (uint32_t b = 0; b < B; b++) v[b] -= lf[k][i][b] * xs[k][b];
      for (uint32_t b = 0; b < B; b++) xs[i][b] = v[b] * rd[i][b];
    }
    for (uint32_t b = 0; b < nb; b++)
      if (pd[b])
        for (uint32_t i = 0; i < p; i++) x[size_t(b) * p + i] = xs[i][b];
  }
  if (dinv) {
    // diag(H^-1)[i] = sum over r >= i of (L^-1)[r][i]^2
    for (uint32_t i = 0; i < p; i++) {
      double sum[B];
      for (uint32_t b = 0; b < B; b++) sum[b] = 0.0;
      for (uint32_t r = i; r < p; r++) {
        for (uint32_t b = 0; b < B; b++) v[b] = r == i ? 1.0 : 0.0;
        for (uint32_t k = i; k < r; k++)
          for (uint32_t b = 0; b < B; b++) v[b] -= lf[r][k][b] * y[k][b];
        for (uint32_t b = 0; b < B; b++) {
          y[r][b] = v[b] * rd[r][b];
          sum[b] += y[r][b] * y[r][b];
        }
      }
      for (uint32_t b = 0; b < nb; b++)
        if (pd[b]) dinv[size_t(b) * p + i] = sum[b];
    }
  }
}
}  // namespace

extern "C" {

int mf_expr_set_create(uint32_t n_names, const char* const* names, uint32_t n_exprs, const char* const* exprs,
                       mf_expr_set** out) {
  if (!out || (n_names && !names) || (n_exprs && !exprs)) return fail(MF_ERR_INVALID, "null argument");
  *out = nullptr;
  std::vector<std::string> nm;
  for (uint32_t i = 0; i < n_names; i++) nm.push_back(names[i] ? names[i] : "");
  try {
    auto set = std::make_unique<mf_expr_set>(nm);
    for (uint32_t i = 0; i < n_exprs; i++) set->roots.push_back(set->dag.parse(exprs[i] ? exprs[i] : ""));
    *out = set.release();
  } catch (const std::exception& e) {
    return fail(MF_ERR_PARSE, e.what());
  }
  return MF_OK;
}

int mf_expr_set_eval(const mf_expr_set* set, uint32_t n_rows, const double* values, double* out) {
  if (!set || (n_rows && (!out || (set->n_names && !values)))) return fail(MF_ERR_INVALID, "null argument");
  std::vector<double> v;
  const size_t ne = set->roots.size();
  for (uint32_t r = 0; r < n_rows; r++) {
    set->dag.eval_all(values + size_t(r) * set->n_names, set->n_names, v);
    for (size_t i = 0; i < ne; i++) out[size_t(r) * ne + i] = v[set->roots[i]];
  }
  return MF_OK;
}

int mf_expr_set_free(mf_expr_set* set) {
  delete set;
  return MF_OK;
}

int mf_spd_solve_batch(uint32_t n, uint32_t p, const double* h, const double* g, double* x, double* dinv,
                       unsigned char* ok) {
  if (p == 0 || p > 64) return fail(MF_ERR_INVALID, "matrix order must be 1 to 64");
  if (n && (!h || !ok || (!g) != (!x))) return fail(MF_ERR_INVALID, "null argument");
  if (p <= kSpdLaneOrder) {
    for (uint32_t t = 0; t < n; t += kSpdLanes) {
      const uint32_t nb = std::min<uint32_t>(kSpdLanes, n - t);
      spd_lanes(nb, p, h + size_t(t) * p * p, g ? g + size_t(t) * p : nullptr, x ? x + size_t(t) * p : nullptr,
                dinv ? dinv + size_t(t) * p : nullptr, ok + t);
    }
    return MF_OK;
  }
  // larger orders: one matrix at a time. lf: lower Cholesky factor (row
  // stride 64); rd[i] = 1 / L[i][i]
  double lf[64 * 64], rd[64], y[64];
  for (uint32_t t = 0; t < n; t++) {
    const double* a = h + size_t(t) * p * p;
    bool pd = true;
    for (uint32_t i = 0; i < p && pd; i++) {
      double* li = lf + i * 64;
      for (uint32_t j = 0; j < i; j++) {
        const double* lj = lf + j * 64;
        double v = a[i * p + j];
        for (uint32_t k = 0; k < j; k++) v -= li[k] * lj[k];
        li[j] = v * rd[j];
      }
      double v = a[i * p + i];
      for (uint32_t k = 0; k < i; k++) v -= li[k] * li[k];
      if (!(v > 0.0)) {
        pd = false;
        break;
      }
      li[i] = std::sqrt(v);
      rd[i] = 1.0 / li[i];
    }
    ok[t] = pd ? 1 : 0;
    if (!pd) continue;
    if (g) {
      const double* gt = g + size_t(t) * p;
      double* xt = x + size_t(t) * p;
      for (uint32_t i = 0; i < p; i++) {
        double v = gt[i];
        for (uint32_t k = 0; k < i; k++) v -= lf[i * 64 + k] * y[k];
        y[i] = v * rd[i];
      }
      for (uint32_t i = p; i-- > 0;) {
        double v = y[i];
        for (uint32_t k = i + 1; k < p; k++) v -= lf[k * 64 + i] * xt[k];
        xt[i] = v * rd[i];
      }
    }
    if (dinv) {
      // diag(H^-1)[i] = sum over r >= i of (L^-1)[r][i]^2; column i of L^-1 by forward substitution
      double* dt = dinv + size_t(t) * p;
      for (uint32_t i = 0; i < p; i++) {
        double sum = 0.0;
        for (uint32_t r = i; r < p; r++) {
          double v = r == i ? 1.0 : 0.0;
          for (uint32_t k = i; k < r; k++) v -= lf[r * 64 + k] * y[k];
          y[r] = v * rd[r];
          sum += y[r] * y[r];
        }
        dt[i] = sum;
      }
    }
  }
  return MF_OK;
}

int mf_splitmix_seed_rows(uint64_t seed, uint32_t nrows, uint32_t* out) {
  if (!out && nrows) return fail(MF_ERR_INVALID, "null argument");
  for (uint32_t r = 0; r < nrows; r++) {
    uint64_t sm = (seed & 0xffffffffULL) * (1ULL << 32) + r;
    for (int k = 0; k < 4; k++) {
      uint64_t z = (sm += 0x9e3779b97f4a7c15ULL);
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
      out[uint64_t(k) * nrows + r] = uint32_t((z ^ (z >> 31)) >> 32);
    }
  }
  return MF_OK;
}

int mf_seed_rows(uint64_t seed, uint32_t nrows, uint32_t* out) {
  if (!out && nrows) return fail(MF_ERR_INVALID, "null argument");
  // Splitmix64 seeding of four 32-bit words (upper halves), then xoshiro128++
  // jumps by 2^64 steps between rows (published jump polynomial).
  uint64_t sm = seed;
  auto splitmix = [&sm]() {
    uint64_t z = (sm += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
  };
  uint32_t st[4];
  for (int k = 0; k < 4; k++) st[k] = uint32_t(splitmix() >> 32);
  auto rotl = [](uint32_t x, int k) { return (x << k) | (x >> (32 - k)); };
  auto next = [&](uint32_t* s) {
    const uint32_t t = s[1] << 9;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 11);
  };
  static const uint32_t J[4] = {0x8764000bu, 0xf542d2d3u, 0x6fa035c3u, 0x77f2db5bu};
  for (uint32_t r = 0; r < nrows; r++) {
    for (int k = 0; k < 4; k++) out[uint64_t(k) * nrows + r] = st[k];
    uint32_t a[4] = {0, 0, 0, 0};
    for (int i = 0; i < 4; i++)
      for (int b = 0; b < 32; b++) {
        if (J[i] & (1u << b))
          for (int k = 0; k < 4; k++) a[k] ^= st[k];
        next(st);
      }
    for (int k = 0; k < 4; k++) st[k] = a[k];
  }
  return MF_OK;
}

int mf_generate_partition(uint64_t n, uint32_t max_workitems, uint64_t* nper, uint32_t* nseeds) {
  if (!nper || !nseeds) return fail(MF_ERR_INVALID, "null argument");
  if (max_workitems > 0 && n > max_workitems) {
    *nper = n / max_workitems + 1;
    *nseeds = uint32_t(n / *nper + 1);
  } else {
    *nper = 1;
    *nseeds = uint32_t(std::max<uint64_t>(n, 1));
  }
  return MF_OK;
}

int mf_compile_check(const mf_kernel_desc* d, int* regs, int* spill) {
  mf::LoweredKernel lk;
  int rc = lower_desc(d, lk);
  if (rc) return rc;
  std::shared_ptr<CompiledImage> img;
  rc = compile_source(lk.source, d->name ? d->name : "kernel", img, lk.entry);
  if (rc) return rc;
  if (regs) *regs = img->regs;
  if (spill) *spill = img->spill;
  return MF_OK;
}

int mf_kernel_free(mf_kernel* k) {
  if (!k) return MF_OK;
  if (k->f64) mf_kernel_free(k->f64);
  mf_context* c = k->ctx;
  res_forget(k);
  if (k->lib) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    cudaLibraryUnload(k->lib);
  }
  const bool counted = k->holds_ref;
  delete k;
  if (counted) release_context(c);
  return MF_OK;
}

int mf_kernel_source(const mf_kernel* k, char* buf, size_t len, size_t* needed) {
  if (!k) return fail(MF_ERR_INVALID, "kernel is null");
  const std::string& s = k->lowered.source;
  if (needed) *needed = s.size() + 1;
  if (buf && len) {
    size_t n = std::min(len - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = '\0';
  }
  return MF_OK;
}

int mf_kernel_info(const mf_kernel* k, int* regs, int* spill, int* block, int* vec) {
  if (!k) return fail(MF_ERR_INVALID, "kernel is null");
  if (regs) *regs = k->image ? k->image->regs : -1;
  if (spill) *spill = k->image ? k->image->spill : -1;
  if (block) *block = k->lowered.block;
  if (vec) *vec = k->lowered.vec;
  return MF_OK;
}

int mf_kernel_read_layout(const mf_kernel* k, uint32_t* columns, uint32_t* bytes_per_event, uint32_t* source_columns) {
  if (!k) return fail(MF_ERR_INVALID, "kernel is null");
  const auto& lk = k->lowered;
  const uint32_t cols = uint32_t(lk.prep ? lk.prep_cols.size() : lk.used_inputs.size());
  const uint32_t es = uint32_t(lk.prep ? lk.prep_elem_bytes() : elem_size(k->elem));
  if (columns) *columns = cols;
  if (bytes_per_event) *bytes_per_event = cols * es;
  if (source_columns) *source_columns = uint32_t(lk.source_inputs.size());
  return MF_OK;
}

}  // extern "C"

namespace mfi {

int grid_for(const mf_kernel* k, uint64_t n) {
  const uint64_t per_block =
      k->lowered.pipelined ? uint64_t(k->lowered.tile) : uint64_t(k->lowered.block) * uint64_t(k->lowered.vec);
  const uint64_t need = std::max<uint64_t>(1, (n + per_block - 1) / per_block);
  const uint64_t cap = uint64_t(k->ctx->num_sms) * uint64_t(k->blocks_per_sm);
  return int(std::min(need, cap));
}

// Launches one REDUCE kernel; `out` is a device-visible address for n_outputs
// doubles. `dependent`: the previous operation on the stream is a REDUCE
// launch of this library that writes nothing this launch reads; the grid may
// then start (programmatic dependent launch) while that one finishes, and
// waits for it before it touches the shared scratch.
int launch_reduce(mf_kernel* k, const void* data, uint64_t stride, uint64_t n, const double* params,
                  double* partials, unsigned* counter, double* out, cudaStream_t stream, int grid_cap,
                  bool dependent, unsigned seq) {
  int grid = grid_for(k, n);
  if (grid_cap > 0) grid = std::min(grid, grid_cap);
  // argument struct: parameter-only values evaluated here, pre-rounded for the kernel's arithmetic
  thread_local std::vector<unsigned char> pv;
  pv.assign(k->lowered.args_bytes(), 0);
  try {
    k->lowered.fill_args(params, k->n_params, pv.data());
  } catch (const std::exception& e) {
    return fail(MF_ERR_INVALID, std::string("parameter evaluation: ") + e.what());
  }
  unsigned* status = k->ctx->status;
  void* args[] = {const_cast<void**>(&data), &stride, &n, pv.data(), &partials, &counter, &out, &status, &seq};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(k->lowered.block);
  cfg.dynamicSmemBytes = k->lowered.smem_bytes;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = dependent ? 1 : 0;
  res_yield(k->ctx);
  MF_CUDA_TRY(cudaLaunchKernelExC(&cfg, reinterpret_cast<const void*>(k->fn), args));
  return MF_OK;
}

// Batched evaluations in chunks of up to kChunk: evaluation e of a chunk
// writes its per-block partials to slot e of the context's partial buffer
// (the _part entry, no waiting, no counter), consecutive grids overlapping
// as programmatic dependent launches; one _combine launch per chunk then
// reduces each evaluation's partials in the fixed order of the
// single-evaluation entry. A chunk's first launch waits for everything
// before it on the stream (its slots were the previous chunk's).
int launch_batched(mf_kernel* k, uint32_t count, const void* const* data, const uint64_t* strides,
                   const uint64_t* ns, const double* params, mf_buffer* out) {
  constexpr uint32_t kChunk = 256;
  mf_context* c = k->ctx;
  int maxgrid = 1;
  for (uint32_t i = 0; i < count; i++) maxgrid = std::max(maxgrid, grid_for(k, ns[i]));
  const uint32_t chunk = std::min(count, kChunk);
  const uint64_t pstride = uint64_t(maxgrid) * k->n_outputs;  // float2 per evaluation
  if (c->ring_cap < chunk * pstride) {
    if (c->ring) {
      MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
      cudaFree(c->ring);
    }
    c->ring = nullptr;
    c->ring_cap = 0;
    // sized for a full chunk of this kernel's evaluations at the largest grid
    // the device runs, so that later batches (of any count) allocate nothing
    const uint64_t full = uint64_t(kChunk) * uint64_t(c->num_sms) * uint64_t(k->blocks_per_sm) * k->n_outputs;
    const uint64_t cap = std::max<uint64_t>(chunk * pstride, full);
    MF_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&c->ring), size_t(cap) * sizeof(float2)));
    c->ring_cap = size_t(cap);
  }
  if (c->ring_grids_cap < kChunk) {
    MF_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&c->ring_grids), kChunk * sizeof(unsigned)));
    c->ring_grids_cap = kChunk;
  }
  const size_t ab = k->lowered.args_bytes();
  std::vector<unsigned char> pv(ab, 0);
  std::vector<unsigned> grids(chunk);
  unsigned* status = c->status;
  for (uint32_t first = 0; first < count; first += chunk) {
    const uint32_t m = std::min(chunk, count - first);
    for (uint32_t i = 0; i < m; i++) {
      const uint32_t e = first + i;
      grids[i] = unsigned(grid_for(k, ns[e]));
      try {
        k->lowered.fill_args(params + uint64_t(e) * k->n_params, k->n_params, pv.data());
      } catch (const std::exception& ex) {
        return fail(MF_ERR_INVALID, std::string("parameter evaluation: ") + ex.what());
      }
      const void* d = data[e];
      uint64_t stride = strides[e], n = ns[e];
      float2* slot = c->ring + uint64_t(i) * pstride;
      void* args[] = {const_cast<void**>(&d), &stride, &n, pv.data(), &slot, &status};
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(grids[i]);
      cfg.blockDim = dim3(k->lowered.block);
      cfg.dynamicSmemBytes = k->lowered.smem_bytes;
      cfg.stream = c->stream;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      attr[0].val.programmaticStreamSerializationAllowed = 1;
      cfg.attrs = attr;
      cfg.numAttrs = i > 0 ? 1 : 0;
      res_yield(k->ctx);
      MF_CUDA_TRY(cudaLaunchKernelExC(&cfg, reinterpret_cast<const void*>(k->fn_part), args));
    }
    // the chunk's grid sizes: one value when they are all equal (evaluations
    // of one size, the common case), else a copy (pageable source: staged
    // before the call returns) that the combine reads
    const bool one_grid = std::all_of(grids.begin(), grids.begin() + m, [&](unsigned x) { return x == grids[0]; });
    if (!one_grid)
      MF_CUDA_TRY(cudaMemcpyAsync(c->ring_grids, grids.data(), m * sizeof(unsigned), cudaMemcpyHostToDevice,
                                  c->stream));
    const float2* ring = c->ring;
    uint64_t ps = pstride;
    const unsigned* g = one_grid ? nullptr : c->ring_grids;
    unsigned grid_all = grids[0];
    double* o = static_cast<double*>(out->ptr) + uint64_t(first) * k->n_outputs;
    uint32_t mm = m;
    void* cargs[] = {const_cast<float2**>(&ring), &ps, const_cast<unsigned**>(&g), &o, &mm, &grid_all};
    // a programmatic dependent of the chunk's last evaluation (which completes
    // after every earlier one): the combine is resident before that grid ends
    // and waits for it in the kernel (unless the grid table copy sits between)
    cudaLaunchConfig_t ccfg = {};
    ccfg.gridDim = dim3(m);
    ccfg.blockDim = dim3(k->lowered.block);
    ccfg.stream = c->stream;
    cudaLaunchAttribute cattr[1];
    cattr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    cattr[0].val.programmaticStreamSerializationAllowed = 1;
    ccfg.attrs = cattr;
    ccfg.numAttrs = one_grid ? 1 : 0;
    MF_CUDA_TRY(cudaLaunchKernelExC(&ccfg, reinterpret_cast<const void*>(k->fn_combine), cargs));
  }
  return MF_OK;
}

}  // namespace mfi

namespace {
bool all_finite(const double* v, size_t n) {
  for (size_t i = 0; i < n; i++)
    if (!std::isfinite(v[i])) return false;
  return true;
}
}  // namespace

extern "C" int mf_kernel_build(mf_context* c, const mf_kernel_desc* d, mf_kernel** out);

// The native-FP64 build of a double-float REDUCE kernel, made on first use.
static int f64_twin(mf_kernel* k) {
  if (k->f64) return MF_OK;
  mf_kernel_desc d = k->desc->d;
  d.flags |= MF_FLAG_NATIVE_F64;
  return mf_kernel_build(k->ctx, &d, &k->f64);
}

static int reduce_direct(mf_kernel* k, const mf_buffer* in, uint64_t stride, uint64_t n, const double* params,
                         uint32_t n_params, double* sums);
namespace {
int res_reduce(mf_kernel* k, const mf_buffer* in, uint64_t stride, uint64_t n, const double* params, double* sums,
               bool* served);
}
int coalesced_reduce(mf_kernel* k, const mf_buffer* in, uint64_t stride, uint64_t n, const double* params,
                     uint32_t n_params, double* sums);

extern "C" {

int mf_kernel_reduce(mf_kernel* k, const mf_buffer* in, uint64_t stride, uint64_t n, const double* params,
                     uint32_t n_params, double* sums) {
  if (!k || !sums) return fail(MF_ERR_INVALID, "null argument");
  if (k->kind == MF_KERNEL_REDUCE && k->ctx->coalescer && n > 0) {
    if (n_params != k->n_params || (n_params && !params))
      return fail(MF_ERR_INVALID, "parameter count mismatch (" + std::to_string(n_params) + " given, " +
                                      std::to_string(k->n_params) + " expected)");
    int rc = check_layout(k, in, stride, n);
    if (rc) return rc;
    MF_CUDA_TRY(cudaSetDevice(k->ctx->device));
    return coalesced_reduce(k, in, stride, n, params, n_params, sums);
  }
  if (k->kind == MF_KERNEL_REDUCE && k->ctx->res && k->ctx->res_idle_ns && n_params == k->n_params &&
      (params || !n_params) && check_layout(k, in, stride, n) == MF_OK) {
    MF_CUDA_TRY(cudaSetDevice(k->ctx->device));
    bool served = false;
    const int rc = res_reduce(k, in, stride, n, params, sums, &served);
    if (rc || served) return rc;
  }
  return reduce_direct(k, in, stride, n, params, n_params, sums);
}

}  // extern "C"

static int reduce_direct(mf_kernel* k, const mf_buffer* in, uint64_t stride, uint64_t n, const double* params,
                         uint32_t n_params, double* sums) {
  if (!k || !sums) return fail(MF_ERR_INVALID, "null argument");
  if (k->kind != MF_KERNEL_REDUCE) return fail(MF_ERR_INVALID, "kernel is not a REDUCE kernel");
  if (n_params != k->n_params || (n_params && !params))
    return fail(MF_ERR_INVALID, "parameter count mismatch (" + std::to_string(n_params) + " given, " +
                                    std::to_string(k->n_params) + " expected)");
  int rc = check_layout(k, in, stride, n);
  if (rc) return rc;
  mf_context* c = k->ctx;
  if (n == 0) {
    std::fill(sums, sums + k->n_outputs, 0.0);
    return MF_OK;
  }
  MF_CUDA_TRY(cudaSetDevice(c->device));
  const int grid = mfi::grid_for(k, n);
  rc = ensure_scratch(c, size_t(grid) * k->n_outputs, k->n_outputs);
  if (rc) return rc;
  *c->status_host = 0u;
  const void* data = nullptr;
  rc = prepare_input(k, in, stride, &data);
  if (rc) return rc;
  if (++c->sync_seq == 0u) c->sync_seq = 1u;  // 0 means "asynchronous" to the kernel
  rc = mfi::launch_reduce(k, data, stride, n, params, c->partials, c->counter, c->out_dev, c->stream, 0, false,
                          c->sync_seq);
  if (rc) return rc;
  rc = wait_sync_word(c, c->sync_seq);
  if (rc) return rc;
  std::memcpy(sums, c->out_host, k->n_outputs * sizeof(double));
  rc = check_status(c);
  if (rc || !k->desc || all_finite(sums, k->n_outputs)) return rc;
  // A double-float intermediate left the FP32 exponent range (|x| > 3.4e38
  // or a quotient of underflowed values): the same launch in native FP64.
  rc = f64_twin(k);
  if (rc) return rc;
  k->fallbacks++;
  return reduce_direct(k->f64, in, stride, n, params, n_params, sums);
}

// ---------------------------------------------------- resident evaluations --
// A context with resident evaluations on (mf_context_set_resident) watches its
// synchronous REDUCE calls. After kResWarmCalls of them it builds, on a
// background thread, one module holding the per-block work (mf_rbody) of the
// kernels those calls used most, each in a namespace of its own, and a
// resident entry. That grid is launched once (cooperative: all its blocks
// co-resident) and loops: block 0 waits for a request in mapped host memory,
// copies it to device memory and releases the other blocks; every block then
// runs the blocks [blockIdx.x, blockIdx.x + gridDim.x, ...) of the kernel's
// own grid for that request (grid_for, as a launch would), and the block
// that completes the count combines the partials and writes the sums and the
// completion word as the single-evaluation entry does. A request's sums are
// those of a launch of the kernel, bit for bit; what it saves is the launch.
// The grid exits when idle for res_idle_ns, or when asked to (a launch of any
// other work on the device, a kernel of the group freed, the context
// destroyed): block 0 swaps the doorbell to kResExit with a system-scope
// compare-and-swap only while no request is pending, so a posted request is
// never dropped, and the host's compare-and-swap of the next request then
// fails and it launches instead. Every wait on the device is bounded.
constexpr unsigned kResExit = 0xffffffffu;
constexpr size_t kResArgsMax = 2048;  // bytes of a member's argument struct
constexpr unsigned kResWarmCalls = 8;
constexpr size_t kResMaxMembers = 2;  // per-block shared memory: ~19 KB per member
constexpr uint64_t kResMaxEvents = uint64_t(1) << 31;
constexpr int64_t kResHoldNs = 20000000;  // no new grid for 20 ms after one was asked to exit

struct ResReq {  // the generated mfr_req
  uint64_t data, stride, n;
  double* out;
  uint32_t which, grid, seq, pad;
  unsigned char args[kResArgsMax];
};
static_assert(sizeof(ResReq) % 16 == 0, "the request is copied in 16-byte words");
struct ResMail {  // the generated mfr_mail (mapped host memory)
  unsigned seq;   // last posted request; kResExit once the grid has left its loop
  unsigned stop;  // nonzero: leave the loop when idle
  unsigned pad[30];
  ResReq req;
};

struct ResState {
  // warm-up: the REDUCE kernels of the first synchronous calls, with call counts
  std::vector<std::pair<mf_kernel*, unsigned>> seen;
  unsigned calls = 0;
  std::thread builder;
  std::atomic<int> state{0};  // 0 watching, 1 building, 2 ready, 3 unavailable
  std::string error;
  // the module (valid once state == 2)
  std::vector<mf_kernel*> members;
  cudaLibrary_t lib = nullptr;
  cudaKernel_t fn = nullptr;
  int grid = 0, block = 0;
  ResMail* mail = nullptr;  // mapped host memory
  ResMail* mail_dev = nullptr;
  ResReq* req = nullptr;  // device copy of the current request
  unsigned* go = nullptr;
  float2* partials = nullptr;
  unsigned* counter = nullptr;
  cudaStream_t stream = nullptr;
  // the grid (alive and the device's owner table change under g_res_mu;
  // the owning thread also reads alive without it, and another context's
  // start may clear it, hence atomic)
  std::atomic<bool> alive{false};
  unsigned posted = 0;
  std::atomic<int64_t> hold_until{0};
  uint64_t served = 0, grids = 0;
};

namespace {

std::mutex g_res_mu;
mf_context* g_res_owner[64] = {};  // per device: the context whose grid is up
std::atomic<int> g_res_up[64];     // per device: a grid may be up (checked without the lock)

int64_t steady_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

// Asks the grid up on device d (whichever context owns it) to exit once
// idle; called before every other launch of this library on the device.
void res_yield_device(int d) {
  if (d < 0 || d >= 64 || !g_res_up[d].load(std::memory_order_acquire)) return;
  std::lock_guard<std::mutex> lk(g_res_mu);
  mf_context* o = g_res_owner[d];
  if (!o || !o->res || !o->res->alive) return;
  __atomic_store_n(&o->res->mail->stop, 1u, __ATOMIC_RELEASE);
  o->res->hold_until.store(steady_ns() + kResHoldNs);
}

void res_yield(mf_context* c) { res_yield_device(c->device); }

// After the grid left (or was asked to leave) its loop: wait for it and
// release the device.
void res_end(mf_context* c) {
  ResState& r = *c->res;
  cudaStreamSynchronize(r.stream);
  std::lock_guard<std::mutex> lk(g_res_mu);
  r.alive = false;
  if (g_res_owner[c->device] == c) {
    g_res_owner[c->device] = nullptr;
    g_res_up[c->device].store(0, std::memory_order_release);
  }
}

void res_stop(mf_context* c) {
  ResState* r = c->res;
  if (!r || !r->alive) return;
  __atomic_store_n(&r->mail->stop, 1u, __ATOMIC_RELEASE);
  res_end(c);
}

// Drops the module and the warm-up record (the grid stopped first).
void res_drop(mf_context* c) {
  ResState& r = *c->res;
  res_stop(c);
  if (r.builder.joinable()) r.builder.join();
  if (r.stream) cudaStreamSynchronize(r.stream);  // a grid that left while idle may still be finishing
  if (r.lib) cudaLibraryUnload(r.lib);
  if (r.mail) cudaFreeHost(r.mail);
  if (r.req) cudaFree(r.req);
  if (r.go) cudaFree(r.go);
  if (r.partials) cudaFree(r.partials);
  if (r.counter) cudaFree(r.counter);
  if (r.stream) cudaStreamDestroy(r.stream);
  r.lib = nullptr;
  r.fn = nullptr;
  r.mail = r.mail_dev = nullptr;
  r.req = nullptr;
  r.go = r.counter = nullptr;
  r.partials = nullptr;
  r.stream = nullptr;
  r.members.clear();
  r.seen.clear();
  r.calls = 0;
  r.state.store(0);
}

void res_shutdown(mf_context* c) {
  if (!c->res) return;
  res_drop(c);
  delete c->res;
  c->res = nullptr;
}

void res_forget(mf_kernel* k) {
  mf_context* c = k->ctx;
  if (!c || !c->res) return;
  ResState& r = *c->res;
  if (r.builder.joinable()) r.builder.join();
  bool used = std::find(r.members.begin(), r.members.end(), k) != r.members.end();
  for (auto& e : r.seen) used = used || e.first == k;
  if (used) res_drop(c);
}

// The resident module's source: every member's translation unit up to its
// entry points plus mf_rbody, in namespace mfr<i> (its macros undefined after
// it), and the resident entry.
std::string res_source(const std::vector<const mf::LoweredKernel*>& m, int block, int min_blocks = 1) {
  std::ostringstream s;
  s << "// MoreFit CUDA backend: resident evaluations of " << m.size() << " REDUCE kernels\n";
  for (size_t i = 0; i < m.size(); i++) {
    const mf::LoweredKernel& L = *m[i];
    s << "namespace mfr" << i << " {\n" << L.resident_prefix << L.resident_body << "}  // namespace mfr" << i << "\n";
    std::vector<std::string> macros;
    std::istringstream t(L.resident_prefix);
    for (std::string line; std::getline(t, line);)
      if (line.rfind("#define ", 0) == 0) {
        size_t e = 8;
        while (e < line.size() && (std::isalnum((unsigned char)line[e]) || line[e] == '_')) e++;
        macros.push_back(line.substr(8, e - 8));
      }
    for (const auto& x : macros) s << "#undef " << x << "\n";
  }
  s << "typedef unsigned long long mfr_u64;\n"
    << "struct mfr_req { mfr_u64 data, stride, n; double* out; unsigned which, grid, seq, pad; unsigned char args["
    << kResArgsMax << "]; };\n"
    << "struct mfr_mail { unsigned seq; unsigned stop; unsigned pad[30]; mfr_req req; };\n"
    << "#define MFR_EXIT 0xffffffffu\n#define MFR_BLOCK " << block << "\n#define MFR_MINB " << min_blocks << "\n";
  size_t args_max = 8;
  for (const auto* L : m) args_max = std::max(args_max, L->args_bytes());
  s << "#define MFR_WORDS " << (48 + args_max + 3) / 4 << "  // request header (48 bytes) and the largest argument struct\n";
  s << R"CUDA(__device__ __forceinline__ unsigned mfr_ld_acq_sys(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned mfr_ld_rlx_sys(const unsigned* p) {
  unsigned v;
  asm volatile("ld.relaxed.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned mfr_ld_acq_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void mfr_st_rel_gpu(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned mfr_cas_sys(unsigned* p, unsigned cmp, unsigned val) {
  unsigned old;
  asm volatile("atom.acq_rel.sys.global.cas.b32 %0, [%1], %2, %3;" : "=r"(old) : "l"(p), "r"(cmp), "r"(val) : "memory");
  return old;
}
__device__ __forceinline__ mfr_u64 mfr_now() {
  mfr_u64 t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// status[0] bit 8: a block gave up waiting for block 0 (the grid then leaves).
extern "C" __global__ void __launch_bounds__(MFR_BLOCK, MFR_MINB) mf_resident(mfr_mail* mail, mfr_req* req, unsigned* go,
                                                                   float2* partials, unsigned* counter,
                                                                   unsigned* status, mfr_u64 idle_ns) {
  __shared__ unsigned mfr_v;
  __shared__ __align__(16) unsigned mfr_rq[MFR_WORDS];
  unsigned seen = 0u;
  for (;;) {
    if (threadIdx.x == 0) {
      const mfr_u64 t0 = mfr_now();
      unsigned v = seen;
      if (blockIdx.x == 0) {
        // the host's doorbell; idle (or asked to stop): leave, unless a request
        // was posted meanwhile (the compare-and-swap then fails and returns it)
        for (unsigned it = 0;; it++) {
          v = mfr_ld_acq_sys(&mail->seq);
          if (v != seen) break;
          if ((it & 3u) == 3u && (mfr_ld_rlx_sys(&mail->stop) != 0u || mfr_now() - t0 > idle_ns)) {
            const unsigned o = mfr_cas_sys(&mail->seq, seen, MFR_EXIT);
            v = o == seen ? MFR_EXIT : o;
            break;
          }
          __nanosleep(32);
        }
      } else {
        // block 0's release of the request; block 0 leaves after idle_ns at
        // most and releases the exit the same way
        for (unsigned it = 0;; it++) {
          v = mfr_ld_acq_gpu(go);
          if (v != seen) break;
          if ((it & 63u) == 63u && mfr_now() - t0 > idle_ns + 2000000000ull) {
            atomicOr(status, 8u);
            v = MFR_EXIT;
            break;
          }
          __nanosleep(32);
        }
      }
      mfr_v = v;
    }
    __syncthreads();
    const unsigned v = mfr_v;
    if (blockIdx.x == 0) {
      if (v != MFR_EXIT) {
        const uint4* src = reinterpret_cast<const uint4*>(&mail->req);
        uint4* dst = reinterpret_cast<uint4*>(req);
        for (unsigned q = threadIdx.x; q < (MFR_WORDS + 3) / 4; q += MFR_BLOCK) dst[q] = __ldcv(src + q);
        __threadfence();
      }
      __syncthreads();
      if (threadIdx.x == 0) mfr_st_rel_gpu(go, v);
    }
    __syncthreads();
    if (v == MFR_EXIT) return;
    seen = v;
    // the request's header and argument struct, staged in shared memory by
    // the first warps: loads of the same words by every thread of the grid
    // would all go to one L2 slice
    for (unsigned w = threadIdx.x; w < MFR_WORDS; w += MFR_BLOCK)
      mfr_rq[w] = __ldcg(reinterpret_cast<const unsigned*>(req) + w);
    __syncthreads();
    const mfr_u64* h64 = reinterpret_cast<const mfr_u64*>(mfr_rq);
    const void* data = reinterpret_cast<const void*>(h64[0]);
    const mfr_u64 stride = h64[1], n = h64[2];
    double* out = reinterpret_cast<double*>(h64[3]);
    const unsigned which = mfr_rq[8], grid = mfr_rq[9], seq = mfr_rq[10];
    switch (which) {
)CUDA";
  for (size_t i = 0; i < m.size(); i++) {
    const std::string ns = "mfr" + std::to_string(i);
    s << "    case " << i << ": {\n"
      << "      const " << ns << "::mf_args& A = *reinterpret_cast<const " << ns << "::mf_args*>(mfr_rq + 12);\n"
      << "      for (unsigned vb = blockIdx.x; vb < grid; vb += gridDim.x) {\n"
      << "        __syncthreads();\n"
      << "        " << ns << "::mf_rbody(static_cast<const " << m[i]->resident_data_type
      << "*>(data), stride, n, A, partials, counter, out, status, seq, vb, grid);\n"
      << "      }\n      break;\n    }\n";
  }
  s << "    default: break;\n    }\n  }\n}\n";
  return s.str();
}

// Background build of the module for `members` (sets state 2, or 3 with error).
void res_build(mf_context* c, std::vector<mf_kernel*> members) {
  ResState& r = *c->res;
  auto give_up = [&](const std::string& why) {
    r.error = why;
    r.state.store(3, std::memory_order_release);
  };
  if (cudaSetDevice(c->device) != cudaSuccess) return give_up("cudaSetDevice");
  const int block = members[0]->lowered.block;
  size_t part = 0;
  for (mf_kernel* k : members)
    part = std::max(part, size_t(c->num_sms) * size_t(k->blocks_per_sm) * size_t(k->n_outputs));
  std::vector<const mf::LoweredKernel*> lowered;
  for (mf_kernel* k : members) lowered.push_back(&k->lowered);
  int member_spill = 0, want = 1;
  for (mf_kernel* k : members) {
    member_spill = std::max(member_spill, k->image ? k->image->spill : 0);
    want = std::max(want, k->blocks_per_sm);
  }
  // as many resident blocks per SM as the member that launches the most
  // (fewer make its blocks run in rounds): the largest count down from there
  // whose register cap spills no more than the kernels themselves
  std::shared_ptr<CompiledImage> img;
  for (int mb = want; mb >= 1 && !img; mb--)
    if (compile_source(res_source(lowered, block, mb), "mf_resident", img, "mf_resident") != MF_OK ||
        img->spill > member_spill)
      img.reset();
  if (!img) return give_up("the resident module spills more than its kernels");
  if (cudaLibraryLoadData(&r.lib, img->cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess ||
      cudaLibraryGetKernel(&r.fn, r.lib, "mf_resident") != cudaSuccess)
    return give_up("loading the resident module");
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, reinterpret_cast<const void*>(r.fn), block, 0) !=
          cudaSuccess ||
      nb < 1)
    return give_up("the resident entry does not fit on an SM");
  r.grid = c->num_sms * std::min(nb, want);
  r.block = block;
  if (cudaHostAlloc(reinterpret_cast<void**>(&r.mail), sizeof(ResMail), cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer(reinterpret_cast<void**>(&r.mail_dev), r.mail, 0) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void**>(&r.req), sizeof(ResReq)) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void**>(&r.go), sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void**>(&r.counter), sizeof(unsigned)) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void**>(&r.partials), std::max<size_t>(part, 1) * sizeof(float2)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&r.stream, cudaStreamNonBlocking) != cudaSuccess)
    return give_up("resident scratch allocation");
  std::memset(r.mail, 0, sizeof(ResMail));
  r.members = std::move(members);
  r.state.store(2, std::memory_order_release);
}

// Launches the grid (the device's previous owner gone): false when another
// context's grid holds the device or the launch failed.
bool res_start(mf_context* c) {
  ResState& r = *c->res;
  r.mail->seq = 0u;
  r.mail->stop = 0u;
  r.posted = 0u;
  {
    std::lock_guard<std::mutex> lk(g_res_mu);
    mf_context*& o = g_res_owner[c->device];
    if (o && o != c) {
      // another context's grid: still up unless it has left its loop (idle);
      // its owner learns that from its next post
      if (__atomic_load_n(&o->res->mail->seq, __ATOMIC_ACQUIRE) != kResExit) return false;
      o->res->alive = false;
    }
    o = c;
    g_res_up[c->device].store(1, std::memory_order_release);
    r.alive = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(unsigned(r.grid));
  cfg.blockDim = dim3(unsigned(r.block));
  cfg.stream = r.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  ResMail* mail = r.mail_dev;
  ResReq* req = r.req;
  unsigned* go = r.go;
  float2* partials = r.partials;
  unsigned* counter = r.counter;
  unsigned* status = c->status;
  unsigned long long idle = c->res_idle_ns;
  void* args[] = {&mail, &req, &go, &partials, &counter, &status, &idle};
  if (cudaMemsetAsync(r.go, 0, sizeof(unsigned), r.stream) != cudaSuccess ||
      cudaMemsetAsync(r.counter, 0, sizeof(unsigned), r.stream) != cudaSuccess ||
      cudaLaunchKernelExC(&cfg, reinterpret_cast<const void*>(r.fn), args) != cudaSuccess) {
    cudaGetLastError();
    res_end(c);
    r.state.store(3);
    r.error = "cooperative launch of the resident grid failed";
    return false;
  }
  r.grids++;
  return true;
}

// One synchronous evaluation through the resident grid. *served false: not
// served, nothing changed (the caller launches as usual).
int res_reduce(mf_kernel* k, const mf_buffer* in, uint64_t stride, uint64_t n, const double* params, double* sums,
               bool* served) {
  *served = false;
  mf_context* c = k->ctx;
  ResState& r = *c->res;
  if (k->lowered.resident_body.empty() || k->lowered.args_bytes() > kResArgsMax || n == 0 || n > kResMaxEvents)
    return MF_OK;
  const int st = r.state.load(std::memory_order_acquire);
  if (st == 0) {
    auto it = std::find_if(r.seen.begin(), r.seen.end(), [&](const auto& e) { return e.first == k; });
    if (it != r.seen.end())
      it->second++;
    else if (r.seen.empty() || r.seen[0].first->lowered.block == k->lowered.block)
      r.seen.emplace_back(k, 1u);
    if (++r.calls >= kResWarmCalls) {
      auto by_use = r.seen;
      std::stable_sort(by_use.begin(), by_use.end(), [](const auto& a, const auto& b) { return a.second > b.second; });
      std::vector<mf_kernel*> members;
      for (size_t i = 0; i < by_use.size() && i < kResMaxMembers; i++) members.push_back(by_use[i].first);
      r.state.store(1);
      r.builder = std::thread(res_build, c, std::move(members));
    }
    return MF_OK;
  }
  if (st != 2) return MF_OK;
  const auto mit = std::find(r.members.begin(), r.members.end(), k);
  if (mit == r.members.end()) return MF_OK;
  // the prepared copy must be current (a launch makes it) and nothing may be
  // pending on the context's stream (it could write what this reads)
  const void* data = in->ptr;
  if (k->lowered.prep) {
    data = nullptr;
    for (const auto& x : in->derived)
      if (x.key == k->prep_key && x.gen == in->gen && x.stride == stride) data = x.ptr;
    if (!data) return MF_OK;
  }
  if (cudaStreamQuery(c->stream) != cudaSuccess) {
    cudaGetLastError();
    return MF_OK;
  }
  if (r.alive && __atomic_load_n(&r.mail->stop, __ATOMIC_ACQUIRE)) {
    res_end(c);  // asked to make room (another launch on the device): it leaves now, idle
    return MF_OK;
  }
  if (!r.alive) {
    if (steady_ns() < r.hold_until.load()) return MF_OK;
    if (!res_start(c)) return MF_OK;
  }
  int rc = ensure_scratch(c, 0, k->n_outputs);
  if (rc) return rc;
  ResReq& q = r.mail->req;
  q.data = reinterpret_cast<uint64_t>(data);
  q.stride = stride;
  q.n = n;
  q.out = c->out_dev;
  q.which = uint32_t(mit - r.members.begin());
  q.grid = uint32_t(mfi::grid_for(k, n));
  if (++c->sync_seq == 0u) c->sync_seq = 1u;
  const unsigned seq = c->sync_seq;
  q.seq = seq;
  try {
    k->lowered.fill_args(params, k->n_params, q.args);
  } catch (const std::exception& e) {
    return fail(MF_ERR_INVALID, std::string("parameter evaluation: ") + e.what());
  }
  *c->status_host = 0u;
  unsigned expected = r.posted;
  unsigned desired = r.posted + 1u;
  if (desired == kResExit || desired == 0u) desired = 1u;
  if (!__atomic_compare_exchange_n(&r.mail->seq, &expected, desired, false, __ATOMIC_RELEASE, __ATOMIC_RELAXED)) {
    res_end(c);  // the grid left its loop; launch instead
    return MF_OK;
  }
  r.posted = desired;
  *served = true;
  // completion word; the grid's waits are bounded, so is this one
  const int64_t t0 = steady_ns();
  for (unsigned spins = 0; __atomic_load_n(c->status_host + 1, __ATOMIC_ACQUIRE) != seq; spins++) {
    if ((spins & 1023u) == 0u && steady_ns() - t0 > int64_t(10) * 1000000000) {
      __atomic_store_n(&r.mail->stop, 1u, __ATOMIC_RELEASE);
      res_end(c);
      return fail(MF_ERR_TIMEOUT, "a resident evaluation did not complete");
    }
  }
  std::memcpy(sums, c->out_host, k->n_outputs * sizeof(double));
  r.served++;
  rc = check_status(c);
  if (rc || !k->desc || all_finite(sums, k->n_outputs)) return rc;
  rc = f64_twin(k);
  if (rc) return rc;
  k->fallbacks++;
  return reduce_direct(k->f64, in, stride, n, params, k->n_params, sums);
}

}  // namespace

namespace mfi {
void resident_yield_device(int device) { res_yield_device(device); }
}  // namespace mfi

extern "C" {

int mf_context_set_resident(mf_context* c, uint32_t idle_us) {
  if (!c) return fail(MF_ERR_INVALID, "null context");
  if (idle_us == 0) {
    if (c->res) res_drop(c);
    c->res_idle_ns = 0;
    return MF_OK;
  }
  int atomics = 0, coop = 0;
  MF_CUDA_TRY(cudaDeviceGetAttribute(&atomics, cudaDevAttrHostNativeAtomicSupported, c->device));
  MF_CUDA_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device));
  if (!atomics || !coop)
    return fail(MF_ERR_UNSUPPORTED, "resident evaluations need host-native atomics and cooperative launches");
  if (!c->res) c->res = new ResState();
  c->res_idle_ns = uint64_t(idle_us) * 1000u;
  return MF_OK;
}

int mf_compile_check_resident(const mf_kernel_desc* const* descs, uint32_t count, int* regs, int* spill,
                              char* source, size_t len) {
  if (!descs || count == 0 || count > kResMaxMembers) return fail(MF_ERR_INVALID, "one or two kernel descriptions");
  std::vector<mf::LoweredKernel> lk(count);
  std::vector<const mf::LoweredKernel*> ptrs;
  for (uint32_t i = 0; i < count; i++) {
    if (!descs[i] || descs[i]->kind != MF_KERNEL_REDUCE) return fail(MF_ERR_INVALID, "REDUCE kernels only");
    int rc = lower_desc(descs[i], lk[i]);
    if (rc) return rc;
    if (lk[i].resident_body.empty()) return fail(MF_ERR_UNSUPPORTED, "kernel has no resident form");
    if (lk[i].block != lk[0].block) return fail(MF_ERR_INVALID, "members differ in block size");
    ptrs.push_back(&lk[i]);
  }
  const std::string src = res_source(ptrs, lk[0].block);
  if (source && len) {
    const size_t n = std::min(len - 1, src.size());
    std::memcpy(source, src.data(), n);
    source[n] = '\0';
  }
  std::shared_ptr<CompiledImage> img;
  int rc = compile_source(src, "mf_resident", img, "mf_resident");
  if (rc) return rc;
  if (regs) *regs = img->regs;
  if (spill) *spill = img->spill;
  return MF_OK;
}

int mf_context_resident_stats(const mf_context* c, int* state, uint64_t* grids, uint64_t* served, int* blocks) {
  if (!c) return fail(MF_ERR_INVALID, "null context");
  const ResState* r = c->res;
  if (blocks) *blocks = r && r->state.load() == 2 ? r->grid : 0;
  if (state) *state = r ? r->state.load() : -1;
  if (grids) *grids = r ? r->grids : 0;
  if (served) *served = r ? r->served : 0;
  return MF_OK;
}

}  // extern "C"

extern "C" {

int mf_kernel_reduce_async(mf_kernel* k, const mf_buffer* in, uint64_t stride, uint64_t n, const double* params,
                           uint32_t n_params, mf_buffer* out, uint64_t out_index) {
  if (!k || !out) return fail(MF_ERR_INVALID, "null argument");
  if (k->kind != MF_KERNEL_REDUCE) return fail(MF_ERR_INVALID, "kernel is not a REDUCE kernel");
  if (n_params != k->n_params || (n_params && !params)) return fail(MF_ERR_INVALID, "parameter count mismatch");
  int rc = check_layout(k, in, stride, n);
  if (rc) return rc;
  if ((out_index + 1) * k->n_outputs * sizeof(double) > out->size)
    return fail(MF_ERR_INVALID, "output buffer too small for out_index");
  if (n == 0) return fail(MF_ERR_INVALID, "no events");
  mf_context* c = k->ctx;
  MF_CUDA_TRY(cudaSetDevice(c->device));
  const int grid = mfi::grid_for(k, n);
  rc = ensure_scratch(c, size_t(grid) * k->n_outputs, k->n_outputs);
  if (rc) return rc;
  double* dst = static_cast<double*>(out->ptr) + out_index * k->n_outputs;
  const void* data = nullptr;
  rc = prepare_input(k, in, stride, &data);
  if (rc) return rc;
  return mfi::launch_reduce(k, data, stride, n, params, c->partials, c->counter, dst, c->stream, 0);
}

int mf_kernel_reduce_many(mf_kernel* k, uint32_t count, const mf_buffer* const* inputs, const uint64_t* strides,
                          const uint64_t* ns, const double* params, uint32_t n_params, mf_buffer* out) {
  if (!k || !inputs || !strides || !ns || !out || (n_params && !params)) return fail(MF_ERR_INVALID, "null argument");
  if (k->kind != MF_KERNEL_REDUCE) return fail(MF_ERR_INVALID, "kernel is not a REDUCE kernel");
  if (n_params != k->n_params) return fail(MF_ERR_INVALID, "parameter count mismatch");
  if (uint64_t(count) * k->n_outputs * sizeof(double) > out->size)
    return fail(MF_ERR_INVALID, "output buffer smaller than count x outputs");
  for (uint32_t i = 0; i < count; i++) {
    int rc = check_layout(k, inputs[i], strides[i], ns[i]);
    if (rc) return rc;
    if (ns[i] == 0) return fail(MF_ERR_INVALID, "launch with no events");
  }
  mf_context* c = k->ctx;
  MF_CUDA_TRY(cudaSetDevice(c->device));
  int maxgrid = 1;
  for (uint32_t i = 0; i < count; i++) maxgrid = std::max(maxgrid, mfi::grid_for(k, ns[i]));
  int rc = ensure_scratch(c, size_t(maxgrid) * k->n_outputs, k->n_outputs);
  if (rc) return rc;
  // Prepared inputs first, then the evaluations back to back: each after the
  // first may overlap its predecessor's tail (it reads only its own input).
  // A buffer that appears with two column strides in one batch would have its
  // prepared copy remade between uses: prepare and launch one by one.
  bool one_by_one = false;
  if (k->lowered.prep && count <= 64) {  // small batches: a scan, no allocation
    for (uint32_t i = 0; i < count && !one_by_one; i++)
      for (uint32_t j = 0; j < i && !one_by_one; j++) one_by_one = inputs[j] == inputs[i] && strides[j] != strides[i];
  } else if (k->lowered.prep) {
    std::map<const mf_buffer*, uint64_t> layout;
    for (uint32_t i = 0; i < count && !one_by_one; i++) {
      auto [it, fresh] = layout.emplace(inputs[i], strides[i]);
      one_by_one = !fresh && it->second != strides[i];
    }
  }
  std::vector<const void*> data(count, nullptr);
  for (uint32_t i = 0; i < count && !one_by_one; i++) {
    rc = prepare_input(k, inputs[i], strides[i], &data[i]);
    if (rc) return rc;
  }
  if (!one_by_one && count > 1) return mfi::launch_batched(k, count, data.data(), strides, ns, params, out);
  for (uint32_t i = 0; i < count; i++) {
    if (one_by_one) {
      rc = prepare_input(k, inputs[i], strides[i], &data[i]);
      if (rc) return rc;
    }
    double* dst = static_cast<double*>(out->ptr) + uint64_t(i) * k->n_outputs;
    rc = mfi::launch_reduce(k, data[i], strides[i], ns[i], params + uint64_t(i) * n_params, c->partials, c->counter,
                            dst, c->stream, 0, i > 0 && !one_by_one);
    if (rc) return rc;
  }
  return MF_OK;
}

int mf_columns_sum(const mf_buffer* buf, int elem, uint32_t ncols, uint64_t n, uint64_t stride, double* sums) {
  if (!buf || !buf->ptr || (!sums && ncols)) return fail(MF_ERR_INVALID, "null argument");
  if (elem != MF_F64 && elem != MF_F32) return fail(MF_ERR_INVALID, "element type must be MF_F64 or MF_F32");
  if (ncols == 0) return MF_OK;
  if (stride < n) return fail(MF_ERR_INVALID, "column stride smaller than the number of events");
  if (uint64_t(ncols) * stride * elem_size(elem) > buf->size)
    return fail(MF_ERR_INVALID, "buffer smaller than ncols x stride");
  if (n == 0) {
    std::fill(sums, sums + ncols, 0.0);
    return MF_OK;
  }
  mf_context* c = buf->ctx;
  MF_CUDA_TRY(cudaSetDevice(c->device));
  const int rows = mfi::columns_sum_partials(n, c->num_sms);
  int rc = ensure_scratch(c, size_t(rows) * ncols, ncols);
  if (rc) return rc;
  rc = mfi::columns_sum_launch(buf->ptr, elem, stride, n, ncols, c->partials, c->counter, c->out_dev, c->stream,
                               c->num_sms);
  if (rc) return rc;
  MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
  std::memcpy(sums, c->out_host, ncols * sizeof(double));
  return MF_OK;
}

int mf_context_stream(mf_context* c, void** stream) {
  if (!c || !stream) return fail(MF_ERR_INVALID, "null argument");
  *stream = c->stream;
  return MF_OK;
}

int mf_kernel_reduce_segments(mf_kernel* k, const mf_buffer* in, uint64_t stride, uint32_t nseg,
                              const uint64_t* seg_begin, const uint32_t* seg_count, const double* params,
                              uint32_t n_params, double* sums) {
  if (!k || !in || !seg_begin || !seg_count || !sums || (n_params && !params))
    return fail(MF_ERR_INVALID, "null argument");
  if (k->kind != MF_KERNEL_REDUCE) return fail(MF_ERR_INVALID, "kernel is not a REDUCE kernel");
  if (n_params != k->n_params) return fail(MF_ERR_INVALID, "parameter count mismatch");
  if (nseg == 0) return MF_OK;
  uint64_t end = 0;
  for (uint32_t s = 0; s < nseg; s++) end = std::max<uint64_t>(end, seg_begin[s] + seg_count[s]);
  int rc = check_layout(k, in, stride, end);
  if (rc) return rc;
  mf_context* c = k->ctx;
  MF_CUDA_TRY(cudaSetDevice(c->device));
  const size_t ab = k->lowered.args_bytes();
  const size_t bytes_begin = size_t(nseg) * 8, bytes_count = (size_t(nseg) * 4 + 15) / 16 * 16,
               bytes_par = size_t(nseg) * ab;
  rc = ensure_stage(c, bytes_begin + bytes_count + bytes_par);
  if (rc) return rc;
  rc = ensure_scratch(c, 0, size_t(nseg) * k->n_outputs);
  if (rc) return rc;
  std::vector<unsigned char> host(bytes_begin + bytes_count + bytes_par, 0);
  std::memcpy(host.data(), seg_begin, bytes_begin);
  std::memcpy(host.data() + bytes_begin, seg_count, size_t(nseg) * 4);
  try {
    k->lowered.fill_args_many(params, n_params, nseg, host.data() + bytes_begin + bytes_count);
  } catch (const std::exception& e) {
    return fail(MF_ERR_INVALID, std::string("parameter evaluation: ") + e.what());
  }
  MF_CUDA_TRY(cudaMemcpyAsync(c->stage_dev, host.data(), host.size(), cudaMemcpyHostToDevice, c->stream));
  char* base = static_cast<char*>(c->stage_dev);
  const uint64_t* d_begin = reinterpret_cast<const uint64_t*>(base);
  const unsigned* d_count = reinterpret_cast<const unsigned*>(base + bytes_begin);
  const void* d_par = base + bytes_begin + bytes_count;
  double* outp = c->out_dev;
  const void* data = nullptr;
  rc = prepare_input(k, in, stride, &data);
  if (rc) return rc;
  void* args[] = {const_cast<void**>(&data), &stride, &d_begin, &d_count, const_cast<void**>(&d_par), &outp};
  res_yield(k->ctx);
  MF_CUDA_TRY(cudaLaunchKernel(reinterpret_cast<const void*>(k->fn_seg), dim3(nseg), dim3(k->lowered.block), args, 0,
                               c->stream));
  MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
  std::memcpy(sums, c->out_host, size_t(nseg) * k->n_outputs * sizeof(double));
  if (!k->desc) return MF_OK;
  // Segments whose double-float sums are non-finite: again in native FP64.
  std::vector<uint32_t> bad;
  for (uint32_t s = 0; s < nseg; s++)
    if (!all_finite(sums + size_t(s) * k->n_outputs, k->n_outputs)) bad.push_back(s);
  if (bad.empty()) return MF_OK;
  rc = f64_twin(k);
  if (rc) return rc;
  k->fallbacks++;
  std::vector<uint64_t> b2(bad.size());
  std::vector<uint32_t> c2(bad.size());
  std::vector<double> p2(bad.size() * n_params), s2(bad.size() * k->n_outputs);
  for (size_t i = 0; i < bad.size(); i++) {
    b2[i] = seg_begin[bad[i]];
    c2[i] = seg_count[bad[i]];
    std::copy(params + size_t(bad[i]) * n_params, params + size_t(bad[i] + 1) * n_params, p2.begin() + i * n_params);
  }
  rc = mf_kernel_reduce_segments(k->f64, in, stride, uint32_t(bad.size()), b2.data(), c2.data(), p2.data(), n_params,
                                 s2.data());
  if (rc) return rc;
  for (size_t i = 0; i < bad.size(); i++)
    std::copy(s2.begin() + i * k->n_outputs, s2.begin() + (i + 1) * k->n_outputs,
              sums + size_t(bad[i]) * k->n_outputs);
  return MF_OK;
}

int mf_kernel_fallback_count(const mf_kernel* k, uint64_t* count) {
  if (!k || !count) return fail(MF_ERR_INVALID, "null argument");
  *count = k->fallbacks;
  return MF_OK;
}

static int kernel_store(mf_kernel* k, const mf_buffer* in, uint64_t in_stride, uint64_t n, const double* params,
                        uint32_t n_params, mf_buffer* out, uint64_t out_stride, bool sync) {
  if (!k || !out) return fail(MF_ERR_INVALID, "null argument");
  if (k->kind != MF_KERNEL_STORE) return fail(MF_ERR_INVALID, "kernel is not a STORE kernel");
  if (n_params != k->n_params || (n_params && !params)) return fail(MF_ERR_INVALID, "parameter count mismatch");
  int rc = check_layout(k, in, in_stride, n);
  if (rc) return rc;
  if (out_stride < n) return fail(MF_ERR_INVALID, "output stride smaller than the number of events");
  if (uint64_t(k->n_outputs) * out_stride * elem_size(k->elem) > out->size)
    return fail(MF_ERR_INVALID, "output buffer smaller than outputs x stride");
  if (n == 0) return MF_OK;
  mf_context* c = k->ctx;
  MF_CUDA_TRY(cudaSetDevice(c->device));
  const uint64_t need = (n + k->lowered.block - 1) / k->lowered.block;
  const int grid = int(std::min<uint64_t>(need, uint64_t(c->num_sms) * k->blocks_per_sm * 4));
  std::vector<double> pv(std::max<uint32_t>(1, k->n_params), 0.0);
  if (k->n_params) std::memcpy(pv.data(), params, k->n_params * sizeof(double));
  const void* data = in->ptr;
  void* outp = out->ptr;
  out->gen++;
  void* args[] = {const_cast<void**>(&data), &in_stride, &n, pv.data(), &outp, &out_stride};
  res_yield(k->ctx);
  MF_CUDA_TRY(cudaLaunchKernel(reinterpret_cast<const void*>(k->fn), dim3(grid), dim3(k->lowered.block), args, 0,
                               c->stream));
  if (sync) MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return MF_OK;
}

int mf_kernel_store(mf_kernel* k, const mf_buffer* in, uint64_t in_stride, uint64_t n, const double* params,
                    uint32_t n_params, mf_buffer* out, uint64_t out_stride) {
  return kernel_store(k, in, in_stride, n, params, n_params, out, out_stride, true);
}

int mf_kernel_store_async(mf_kernel* k, const mf_buffer* in, uint64_t in_stride, uint64_t n, const double* params,
                          uint32_t n_params, mf_buffer* out, uint64_t out_stride) {
  return kernel_store(k, in, in_stride, n, params, n_params, out, out_stride, false);
}

// seeds null: every stream seeded on the device from `splitmix_seed` (the
// state mf_splitmix_seed_rows gives its row), no seed table copied.
static int kernel_generate(mf_kernel* k, const uint32_t* seeds, uint32_t nseeds, uint64_t n, uint64_t nper,
                           const double* params, uint32_t n_params, mf_buffer* out, uint64_t out_stride,
                           uint64_t max_tries, bool sync, uint64_t splitmix_seed = 0) {
  if (!k || !out) return fail(MF_ERR_INVALID, "null argument");
  if (k->kind != MF_KERNEL_GENERATE) return fail(MF_ERR_INVALID, "kernel is not a GENERATE kernel");
  if (n_params != k->n_params || (n_params && !params)) return fail(MF_ERR_INVALID, "parameter count mismatch");
  if (nseeds == 0 || nper == 0) return fail(MF_ERR_INVALID, "no generator threads");
  if (uint64_t(nseeds) * nper < n) return fail(MF_ERR_INVALID, "nseeds x nper does not cover n events");
  if (out_stride < n || uint64_t(k->n_gen_dims) * out_stride * elem_size(k->elem) > out->size)
    return fail(MF_ERR_INVALID, "output buffer smaller than dimensions x stride");
  if (n == 0) return MF_OK;
  mf_context* c = k->ctx;
  MF_CUDA_TRY(cudaSetDevice(c->device));
  if (seeds) {
    int rc = ensure_stage(c, size_t(nseeds) * 4 * sizeof(uint32_t));
    if (rc) return rc;
    MF_CUDA_TRY(cudaMemcpyAsync(c->stage_dev, seeds, size_t(nseeds) * 4 * sizeof(uint32_t), cudaMemcpyHostToDevice,
                                c->stream));
  }
  if (sync) *c->status_host = 0u;
  std::vector<double> pv(std::max<uint32_t>(1, k->n_params), 0.0);
  if (k->n_params) std::memcpy(pv.data(), params, k->n_params * sizeof(double));
  const unsigned* sd = seeds ? static_cast<const unsigned*>(c->stage_dev) : nullptr;
  void* outp = out->ptr;
  out->gen++;
  unsigned* status = c->status;
  unsigned long long mt = max_tries ? max_tries : 1000000000ULL;
  unsigned long long sms = splitmix_seed;
  void* args[] = {&sd, &nseeds, &n, &nper, pv.data(), &outp, &out_stride, &status, &mt, &sms};
  const unsigned grid = (nseeds + k->lowered.block - 1) / k->lowered.block;
  res_yield(k->ctx);
  MF_CUDA_TRY(cudaLaunchKernel(reinterpret_cast<const void*>(k->fn), dim3(grid), dim3(k->lowered.block), args, 0,
                               c->stream));
  if (!sync) return MF_OK;
  MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
  const unsigned st = *c->status_host;
  *c->status_host = 0u;
  if (st) return fail(MF_ERR_TIMEOUT, "generation gave up after max_tries proposals in at least one thread");
  return MF_OK;
}

int mf_kernel_generate(mf_kernel* k, const uint32_t* seeds, uint32_t nseeds, uint64_t n, uint64_t nper,
                       const double* params, uint32_t n_params, mf_buffer* out, uint64_t out_stride,
                       uint64_t max_tries) {
  if (!seeds) return fail(MF_ERR_INVALID, "null argument");
  return kernel_generate(k, seeds, nseeds, n, nper, params, n_params, out, out_stride, max_tries, true);
}

int mf_kernel_generate_splitmix_async(mf_kernel* k, uint64_t seed, uint32_t nstreams, uint64_t n, uint64_t nper,
                                      const double* params, uint32_t n_params, mf_buffer* out, uint64_t out_stride,
                                      uint64_t max_tries) {
  return kernel_generate(k, nullptr, nstreams, n, nper, params, n_params, out, out_stride, max_tries, false, seed);
}

int mf_kernel_generate_async(mf_kernel* k, const uint32_t* seeds, uint32_t nseeds, uint64_t n, uint64_t nper,
                             const double* params, uint32_t n_params, mf_buffer* out, uint64_t out_stride,
                             uint64_t max_tries) {
  if (!seeds) return fail(MF_ERR_INVALID, "null argument");
  return kernel_generate(k, seeds, nseeds, n, nper, params, n_params, out, out_stride, max_tries, false);
}

int mf_kernel_generate_segments(mf_kernel* k, const uint32_t* seeds, uint32_t nthreads, uint32_t threads_per_seg,
                                uint32_t nseg, const uint64_t* seg_begin, const uint32_t* seg_count,
                                const double* seg_params, uint32_t n_params, const double* seg_maxprob,
                                mf_buffer* out, uint64_t out_stride, uint64_t max_tries) {
  if (!k || !seeds || !seg_begin || !seg_count || !seg_maxprob || !out || (n_params && !seg_params))
    return fail(MF_ERR_INVALID, "null argument");
  if (k->kind != MF_KERNEL_GENERATE) return fail(MF_ERR_INVALID, "kernel is not a GENERATE kernel");
  if (n_params != k->n_params) return fail(MF_ERR_INVALID, "parameter count mismatch");
  if (threads_per_seg == 0 || uint64_t(nseg) * threads_per_seg != nthreads)
    return fail(MF_ERR_INVALID, "nthreads must equal nseg x threads_per_seg");
  if (nseg == 0) return MF_OK;
  for (uint32_t s = 0; s < nseg; s++)
    if (seg_begin[s] + seg_count[s] > out_stride)
      return fail(MF_ERR_INVALID, "segment " + std::to_string(s) + " reaches beyond the output stride");
  if (uint64_t(k->n_gen_dims) * out_stride * elem_size(k->elem) > out->size)
    return fail(MF_ERR_INVALID, "output buffer smaller than dimensions x stride");
  mf_context* c = k->ctx;
  MF_CUDA_TRY(cudaSetDevice(c->device));
  const size_t np = std::max<uint32_t>(1, n_params);  // mf_par holds at least one value
  const size_t b_seeds = (size_t(nthreads) * 16 + 15) / 16 * 16, b_begin = size_t(nseg) * 8,
               b_count = (size_t(nseg) * 4 + 15) / 16 * 16, b_par = size_t(nseg) * np * 8, b_max = size_t(nseg) * 8;
  std::vector<unsigned char> host(b_seeds + b_begin + b_count + b_par + b_max, 0);
  std::memcpy(host.data(), seeds, size_t(nthreads) * 16);
  std::memcpy(host.data() + b_seeds, seg_begin, b_begin);
  std::memcpy(host.data() + b_seeds + b_begin, seg_count, size_t(nseg) * 4);
  double* par = reinterpret_cast<double*>(host.data() + b_seeds + b_begin + b_count);
  for (uint32_t s = 0; s < nseg; s++)
    for (uint32_t q = 0; q < n_params; q++) par[size_t(s) * np + q] = seg_params[size_t(s) * n_params + q];
  std::memcpy(host.data() + b_seeds + b_begin + b_count + b_par, seg_maxprob, b_max);
  int rc = ensure_stage(c, host.size());
  if (rc) return rc;
  MF_CUDA_TRY(cudaMemcpyAsync(c->stage_dev, host.data(), host.size(), cudaMemcpyHostToDevice, c->stream));
  char* base = static_cast<char*>(c->stage_dev);
  const unsigned* d_seeds = reinterpret_cast<const unsigned*>(base);
  const uint64_t* d_begin = reinterpret_cast<const uint64_t*>(base + b_seeds);
  const unsigned* d_count = reinterpret_cast<const unsigned*>(base + b_seeds + b_begin);
  const void* d_par = base + b_seeds + b_begin + b_count;
  const double* d_max = reinterpret_cast<const double*>(base + b_seeds + b_begin + b_count + b_par);
  *c->status_host = 0u;
  out->gen++;
  void* outp = out->ptr;
  unsigned* status = c->status;
  unsigned long long mt = max_tries ? max_tries : 1000000000ULL;
  void* args[] = {&d_seeds, &nthreads, &threads_per_seg, &d_begin, &d_count, const_cast<void**>(&d_par), &d_max,
                  &outp, &out_stride, &status, &mt};
  const unsigned grid = (nthreads + k->lowered.block - 1) / k->lowered.block;
  res_yield(k->ctx);
  MF_CUDA_TRY(cudaLaunchKernel(reinterpret_cast<const void*>(k->fn_seg), dim3(grid), dim3(k->lowered.block), args, 0,
                               c->stream));
  MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
  const unsigned st = *c->status_host;
  *c->status_host = 0u;
  if (st) return fail(MF_ERR_TIMEOUT, "generation gave up after max_tries proposals in at least one thread");
  return MF_OK;
}

}  // extern "C"

// ------------------------------------------------- many datasets per launch --
namespace mfi {

constexpr uint64_t kMultiChunk = 2048;  // events per segment of a _multi launch (8 per thread)

struct MultiSeg {  // the generated sources' mf_seg
  const void* data;
  uint64_t stride, first;
  uint32_t count, req, row, pad;
};
static_assert(sizeof(MultiSeg) == 40, "mf_seg layout");

// One evaluation of a multi-dataset launch.
struct MultiItem {
  mf_kernel* k;          // built from the launch's source: its argument layout
  const void* data;      // the columns the kernel reads (prepared when it reads prepared columns)
  uint64_t stride, n;    // n >= 1
  const double* params;  // k->n_params values
};

uint64_t multi_segments(uint64_t n, uint64_t chunk = kMultiChunk) { return std::max<uint64_t>(1, (n + chunk - 1) / chunk); }

size_t round16(size_t b) { return (b + 15) / 16 * 16; }

// Host staging bytes launch_multi needs for `items`: the segment table, one
// argument struct per item, and the per-item segment counts.
size_t multi_table_bytes(const mf_kernel* k, const std::vector<MultiItem>& items, uint64_t chunk = kMultiChunk) {
  uint64_t nseg = 0;
  for (const auto& it : items) nseg += multi_segments(it.n, chunk);
  return round16(size_t(nseg) * sizeof(MultiSeg)) + round16(items.size() * k->lowered.args_bytes()) +
         round16(items.size() * sizeof(unsigned));
}

// Enqueues on c's stream one _multi launch over every segment of every item
// and one _combine launch (one block per item) that writes item e's sums to
// out[e * n_outputs ...] (device-visible memory). Every item's kernel is
// built from k0's source. `host` is staging of multi_table_bytes() bytes that
// stays untouched until the stream has executed the table copy. Segment s of
// an item covers its events [s * chunk, ...): an item's sums depend on
// nothing but its own events, parameters, size and the chunk.
int launch_multi(mf_context* c, mf_kernel* k0, const std::vector<MultiItem>& items, unsigned char* host,
                 double* out, uint64_t chunk = kMultiChunk) {
  if (items.empty()) return MF_OK;
  const size_t ab = k0->lowered.args_bytes();
  uint64_t nseg = 0, pmax = 1;
  for (const auto& it : items) {
    nseg += multi_segments(it.n, chunk);
    pmax = std::max(pmax, multi_segments(it.n, chunk));
  }
  if (nseg > 0x7fffffffu) return fail(MF_ERR_INVALID, "too many segments in one launch");
  const size_t b_seg = round16(size_t(nseg) * sizeof(MultiSeg)), b_args = round16(items.size() * ab);
  const size_t b_grid = round16(items.size() * sizeof(unsigned));
  auto* segs = reinterpret_cast<MultiSeg*>(host);
  unsigned char* args = host + b_seg;
  auto* grids = reinterpret_cast<unsigned*>(host + b_seg + b_args);
  uint64_t q = 0;
  for (size_t e = 0; e < items.size(); e++) {
    const MultiItem& it = items[e];
    const uint64_t ns = multi_segments(it.n, chunk);
    for (uint64_t s = 0; s < ns; s++, q++) {
      const uint64_t first = s * chunk;
      segs[q] = MultiSeg{it.data, it.stride, first, uint32_t(std::min<uint64_t>(chunk, it.n - first)),
                         uint32_t(e), uint32_t(e * pmax + s), 0u};
    }
    grids[e] = unsigned(ns);
    try {
      it.k->lowered.fill_args(it.params, it.k->n_params, args + e * ab);
    } catch (const std::exception& ex) {
      return fail(MF_ERR_INVALID, std::string("parameter evaluation: ") + ex.what());
    }
  }
  int rc = ensure_stage(c, b_seg + b_args + b_grid);
  if (rc) return rc;
  const uint64_t need = uint64_t(items.size()) * pmax * k0->n_outputs;  // float2 partial rows
  if (c->ring_cap < need) {
    if (c->ring) {
      MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
      cudaFree(c->ring);
    }
    c->ring = nullptr;
    c->ring_cap = 0;
    const uint64_t cap = std::max<uint64_t>(need + need / 2, uint64_t(1) << 16);
    MF_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(&c->ring), size_t(cap) * sizeof(float2)));
    c->ring_cap = size_t(cap);
  }
  MF_CUDA_TRY(cudaMemcpyAsync(c->stage_dev, host, b_seg + b_args + b_grid, cudaMemcpyHostToDevice, c->stream));
  char* base = static_cast<char*>(c->stage_dev);
  const void* d_segs = base;
  const void* d_args = base + b_seg;
  const unsigned* d_grids = reinterpret_cast<const unsigned*>(base + b_seg + b_args);
  float2* ring = c->ring;
  void* margs[] = {const_cast<void**>(&d_segs), const_cast<void**>(&d_args), &ring};
  res_yield(k0->ctx);
  MF_CUDA_TRY(cudaLaunchKernel(reinterpret_cast<const void*>(k0->fn_multi), dim3(unsigned(nseg)),
                               dim3(k0->lowered.block), margs, 0, c->stream));
  const float2* cring = ring;
  uint64_t pstride = pmax * k0->n_outputs;
  unsigned count = unsigned(items.size());
  unsigned grid_all = 0;  // unused: per-item counts in d_grids
  void* cargs[] = {const_cast<float2**>(&cring), &pstride, const_cast<unsigned**>(&d_grids), &out, &count,
                   &grid_all};
  MF_CUDA_TRY(cudaLaunchKernel(reinterpret_cast<const void*>(k0->fn_combine), dim3(count), dim3(k0->lowered.block),
                               cargs, 0, c->stream));
  return MF_OK;
}

}  // namespace mfi

// ---------------------------------------------------------------- coalescer --
// Synchronous evaluations from many host threads (each with its own context,
// e.g. one fitter and its CUDABlocks per thread) gathered into shared launches.
namespace {

struct CoalReq {
  mf_kernel* k = nullptr;
  const void* data = nullptr;
  uint64_t stride = 0, n = 0;
  const double* params = nullptr;
  double* sums = nullptr;      // host destination, k->n_outputs doubles
  std::vector<double> owned;   // asynchronous submissions: params, then sums
  std::atomic<int> state{0};   // 0 pending, 1 done, 2 failed
  std::string error;
};

}  // namespace

struct mf_coalescer {
  int device = 0;
  mf_context* ctx = nullptr;  // the dispatch stream and its scratch
  uint32_t max_batch = 256;
  uint32_t window_us = 30;
  std::mutex mu;
  std::condition_variable cv, done_cv;
  std::deque<CoalReq*> pending;
  std::map<uint64_t, std::unique_ptr<CoalReq>> tickets;
  uint64_t next_ticket = 1;
  int clients = 0;
  bool stop = false;
  std::thread worker;
  std::atomic<uint64_t> ticks{0}, evaluations{0};
  std::atomic<uint32_t> max_seen{0};
  double* out_host = nullptr;
  double* out_dev = nullptr;
  size_t out_cap = 0;  // doubles
  unsigned char* tables = nullptr;
  size_t tables_cap = 0;
};

namespace {

// Sets every request of the batch to failed with the current error message.
void coal_fail_all(std::vector<CoalReq*>& batch, const std::string& msg) {
  for (auto* r : batch) {
    r->error = msg;
    r->state.store(2, std::memory_order_release);
  }
}

// Launches one tick: the batch grouped by kernel source (one _multi and one
// _combine launch per group, all on the dispatch stream), then waits for the
// stream and hands each request its sums.
void coal_execute(mf_coalescer* co, std::vector<CoalReq*>& batch) {
  mf_context* c = co->ctx;
  std::map<const CompiledImage*, std::vector<size_t>> groups;
  size_t nout_total = 0;
  for (size_t i = 0; i < batch.size(); i++) {
    groups[batch[i]->k->image.get()].push_back(i);
    nout_total += batch[i]->k->n_outputs;
  }
  std::vector<std::vector<mfi::MultiItem>> items(groups.size());
  size_t table_bytes = 0, g = 0;
  for (auto& [img, idx] : groups) {
    for (size_t i : idx) {
      CoalReq* r = batch[i];
      items[g].push_back(mfi::MultiItem{r->k, r->data, r->stride, r->n, r->params});
    }
    table_bytes += mfi::round16(mfi::multi_table_bytes(items[g][0].k, items[g]));
    g++;
  }
  auto cuda_fail = [&](const char* what, cudaError_t e) {
    coal_fail_all(batch, std::string(what) + ": " + cudaGetErrorString(e));
  };
  if (nout_total > co->out_cap) {
    if (co->out_host) cudaFreeHost(co->out_host);
    co->out_host = nullptr;
    co->out_cap = 0;
    const size_t cap = std::max<size_t>(nout_total * 2, 4096);
    cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&co->out_host), cap * sizeof(double), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&co->out_dev), co->out_host, 0);
    if (e != cudaSuccess) return cuda_fail("cudaHostAlloc", e);
    co->out_cap = cap;
  }
  if (table_bytes > co->tables_cap) {
    if (co->tables) cudaFreeHost(co->tables);
    co->tables = nullptr;
    co->tables_cap = 0;
    const size_t cap = std::max<size_t>(table_bytes * 2, 1 << 16);
    cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&co->tables), cap, cudaHostAllocDefault);
    if (e != cudaSuccess) return cuda_fail("cudaHostAlloc", e);
    co->tables_cap = cap;
  }
  // Each group stages its tables from its own range of the pinned buffer and
  // writes its outputs to its own range of the mapped results; the device
  // stage buffer and partial rows are reused group after group, which stream
  // order makes safe (a group's table copy runs after the previous group's
  // kernels).
  size_t toff = 0, ooff = 0;
  g = 0;
  std::vector<size_t> out_off(batch.size());
  for (auto& [img, idx] : groups) {
    for (size_t j = 0; j < idx.size(); j++) out_off[idx[j]] = ooff + j * batch[idx[0]]->k->n_outputs;
    const int rc = mfi::launch_multi(c, items[g][0].k, items[g], co->tables + toff, co->out_dev + ooff);
    if (rc) {
      // the groups launched before this one still write the mapped results:
      // let them finish before the next tick reuses that memory
      const std::string msg = mf_last_error();
      cudaStreamSynchronize(c->stream);
      return coal_fail_all(batch, msg);
    }
    toff += mfi::round16(mfi::multi_table_bytes(items[g][0].k, items[g]));
    ooff += idx.size() * batch[idx[0]]->k->n_outputs;
    g++;
  }
  const cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_fail("cudaStreamSynchronize", e);
  for (size_t i = 0; i < batch.size(); i++) {
    CoalReq* r = batch[i];
    std::memcpy(r->sums, co->out_host + out_off[i], r->k->n_outputs * sizeof(double));
    r->state.store(1, std::memory_order_release);
  }
  co->ticks++;
  co->evaluations += batch.size();
  uint32_t m = co->max_seen.load();
  while (batch.size() > m && !co->max_seen.compare_exchange_weak(m, uint32_t(batch.size()))) {}
}

void coal_worker(mf_coalescer* co) {
  cudaSetDevice(co->device);
  std::vector<CoalReq*> batch;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(co->mu);
      co->cv.wait(lk, [&] { return co->stop || !co->pending.empty(); });
      if (co->pending.empty()) return;  // stopping, nothing left
      // gather: until every attached context has a request waiting, the batch
      // is full, or the window since this wake-up has passed
      const auto deadline = std::chrono::steady_clock::now() + std::chrono::microseconds(co->window_us);
      while (!co->stop && co->pending.size() < co->max_batch && int(co->pending.size()) < co->clients)
        if (co->cv.wait_until(lk, deadline) == std::cv_status::timeout) break;
      batch.clear();
      while (!co->pending.empty() && batch.size() < co->max_batch) {
        batch.push_back(co->pending.front());
        co->pending.pop_front();
      }
    }
    coal_execute(co, batch);
    { std::lock_guard<std::mutex> lk(co->mu); }
    co->done_cv.notify_all();
  }
}

void coal_push(mf_coalescer* co, CoalReq* r) {
  {
    std::lock_guard<std::mutex> lk(co->mu);
    co->pending.push_back(r);
  }
  co->cv.notify_one();
}

// Waits for request r: a short spin (a tick often completes within it), then blocks.
void coal_wait(mf_coalescer* co, CoalReq* r) {
  const auto t0 = std::chrono::steady_clock::now();
  while (r->state.load(std::memory_order_acquire) == 0) {
    if (std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(50)) {
      std::unique_lock<std::mutex> lk(co->mu);
      co->done_cv.wait(lk, [&] { return r->state.load(std::memory_order_acquire) != 0; });
      break;
    }
  }
}

// Fills a request for kernel k over buffer `in`: the columns it reads (its
// prepared copy, made on the requester's stream) and the requester's stream
// drained, so that the dispatch stream sees every upload and preparation.
int coal_prepare(mf_kernel* k, const mf_buffer* in, uint64_t stride, uint64_t n, CoalReq* r) {
  const void* data = nullptr;
  int rc = prepare_input(k, in, stride, &data);
  if (rc) return rc;
  mf_context* c = k->ctx;
  if (cudaStreamQuery(c->stream) != cudaSuccess) {
    cudaGetLastError();  // cudaErrorNotReady is a state, not an error
    MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
  }
  r->k = k;
  r->data = data;
  r->stride = stride;
  r->n = n;
  return MF_OK;
}

}  // namespace

// mf_kernel_reduce for a context with a coalescer: the evaluation joins the
// coalescer's next tick; a non-finite double-float sum is evaluated again on
// this context in native FP64, not coalesced.
int coalesced_reduce(mf_kernel* k, const mf_buffer* in, uint64_t stride, uint64_t n, const double* params,
                     uint32_t n_params, double* sums) {
  mf_coalescer* co = k->ctx->coalescer;
  CoalReq r;
  int rc = coal_prepare(k, in, stride, n, &r);
  if (rc) return rc;
  r.params = params;
  r.sums = sums;
  coal_push(co, &r);
  coal_wait(co, &r);
  if (r.state.load() == 2) return fail(MF_ERR_CUDA, "coalesced evaluation: " + r.error);
  if (!k->desc || all_finite(sums, k->n_outputs)) return MF_OK;
  rc = f64_twin(k);
  if (rc) return rc;
  k->fallbacks++;
  return reduce_direct(k->f64, in, stride, n, params, n_params, sums);
}

extern "C" {

int mf_kernel_reduce_multi(mf_kernel* k, uint32_t count, const mf_buffer* const* inputs, const uint64_t* strides,
                           const uint64_t* ns, const double* params, uint32_t n_params, mf_buffer* out) {
  if (!k || !inputs || !strides || !ns || !out || (n_params && !params)) return fail(MF_ERR_INVALID, "null argument");
  if (k->kind != MF_KERNEL_REDUCE) return fail(MF_ERR_INVALID, "kernel is not a REDUCE kernel");
  if (n_params != k->n_params) return fail(MF_ERR_INVALID, "parameter count mismatch");
  if (uint64_t(count) * k->n_outputs * sizeof(double) > out->size)
    return fail(MF_ERR_INVALID, "output buffer smaller than count x outputs");
  if (count == 0) return MF_OK;
  mf_context* c = k->ctx;
  MF_CUDA_TRY(cudaSetDevice(c->device));
  std::vector<mfi::MultiItem> items(count);
  for (uint32_t i = 0; i < count; i++) {
    int rc = check_layout(k, inputs[i], strides[i], ns[i]);
    if (rc) return rc;
    if (ns[i] == 0) return fail(MF_ERR_INVALID, "evaluation with no events");
    const void* data = nullptr;
    rc = prepare_input(k, inputs[i], strides[i], &data);
    if (rc) return rc;
    items[i] = mfi::MultiItem{k, data, strides[i], ns[i], params + uint64_t(i) * n_params};
  }
  // pageable staging: cudaMemcpyAsync has copied it when it returns
  std::vector<unsigned char> host(mfi::multi_table_bytes(k, items));
  return mfi::launch_multi(c, k, items, host.data(), static_cast<double*>(out->ptr));
}

int mf_coalescer_create(int device, uint32_t max_batch, uint32_t window_us, mf_coalescer** out) {
  if (!out) return fail(MF_ERR_INVALID, "out is null");
  *out = nullptr;
  auto co = std::make_unique<mf_coalescer>();
  int rc = mf_context_create(device, 0, &co->ctx);
  if (rc) return rc;
  co->device = device;
  co->max_batch = max_batch ? max_batch : 256;
  co->window_us = window_us;
  try {
    co->worker = std::thread(coal_worker, co.get());
  } catch (const std::exception& e) {
    mf_context_destroy(co->ctx);
    return fail(MF_ERR_INVALID, std::string("cannot start the dispatch thread: ") + e.what());
  }
  *out = co.release();
  return MF_OK;
}

int mf_coalescer_destroy(mf_coalescer* co) {
  if (!co) return MF_OK;
  {
    std::lock_guard<std::mutex> lk(co->mu);
    if (co->clients > 0) return fail(MF_ERR_INVALID, "contexts are still attached to the coalescer");
    co->stop = true;
  }
  co->cv.notify_all();
  co->worker.join();
  if (co->out_host) cudaFreeHost(co->out_host);
  if (co->tables) cudaFreeHost(co->tables);
  mf_context_destroy(co->ctx);
  delete co;
  return MF_OK;
}

int mf_context_set_coalescer(mf_context* c, mf_coalescer* co) {
  if (!c) return fail(MF_ERR_INVALID, "null context");
  if (co && co->device != c->device) return fail(MF_ERR_INVALID, "coalescer and context are on different devices");
  if (c->coalescer == co) return MF_OK;
  if (c->coalescer) {
    std::lock_guard<std::mutex> lk(c->coalescer->mu);
    c->coalescer->clients--;
  }
  c->coalescer = co;
  if (co) {
    std::lock_guard<std::mutex> lk(co->mu);
    co->clients++;
  }
  return MF_OK;
}

int mf_coalesced_submit(mf_coalescer* co, mf_kernel* k, const mf_buffer* in, uint64_t stride, uint64_t n,
                        const double* params, uint32_t n_params, uint64_t* ticket) {
  if (!co || !k || !ticket || (n_params && !params)) return fail(MF_ERR_INVALID, "null argument");
  if (k->kind != MF_KERNEL_REDUCE) return fail(MF_ERR_INVALID, "kernel is not a REDUCE kernel");
  if (n_params != k->n_params) return fail(MF_ERR_INVALID, "parameter count mismatch");
  if (k->ctx->device != co->device) return fail(MF_ERR_INVALID, "kernel and coalescer are on different devices");
  int rc = check_layout(k, in, stride, n);
  if (rc) return rc;
  if (n == 0) return fail(MF_ERR_INVALID, "evaluation with no events");
  MF_CUDA_TRY(cudaSetDevice(k->ctx->device));
  auto r = std::make_unique<CoalReq>();
  rc = coal_prepare(k, in, stride, n, r.get());
  if (rc) return rc;
  r->owned.assign(params, params + n_params);
  r->owned.resize(size_t(n_params) + k->n_outputs, 0.0);
  r->params = r->owned.data();
  r->sums = r->owned.data() + n_params;
  CoalReq* raw = r.get();
  {
    std::lock_guard<std::mutex> lk(co->mu);
    *ticket = co->next_ticket++;
    co->tickets.emplace(*ticket, std::move(r));
    co->pending.push_back(raw);
  }
  co->cv.notify_one();
  return MF_OK;
}

int mf_coalesced_poll(mf_coalescer* co, uint64_t ticket, double* sums, int wait) {
  if (!co || !sums) return fail(MF_ERR_INVALID, "null argument");
  CoalReq* r = nullptr;
  {
    std::lock_guard<std::mutex> lk(co->mu);
    auto it = co->tickets.find(ticket);
    if (it == co->tickets.end()) return fail(MF_ERR_INVALID, "unknown ticket");
    r = it->second.get();
  }
  if (r->state.load(std::memory_order_acquire) == 0) {
    if (!wait) return MF_ERR_NOT_READY;
    coal_wait(co, r);
  }
  const int st = r->state.load();
  std::unique_ptr<CoalReq> owned;
  {
    std::lock_guard<std::mutex> lk(co->mu);
    auto it = co->tickets.find(ticket);
    owned = std::move(it->second);
    co->tickets.erase(it);
  }
  if (st == 2) return fail(MF_ERR_CUDA, "coalesced evaluation: " + owned->error);
  std::memcpy(sums, owned->sums, owned->k->n_outputs * sizeof(double));
  return MF_OK;
}

int mf_coalescer_stats(const mf_coalescer* co, uint64_t* ticks, uint64_t* evaluations, uint32_t* max_batch) {
  if (!co) return fail(MF_ERR_INVALID, "null coalescer");
  if (ticks) *ticks = co->ticks.load();
  if (evaluations) *evaluations = co->evaluations.load();
  if (max_batch) *max_batch = co->max_seen.load();
  return MF_OK;
}

}  // extern "C"

// ------------------------------------- ragged segments through the multi entry --
extern "C" int mf_kernel_reduce_segments_chunked(mf_kernel* k, const mf_buffer* in, uint64_t stride, uint32_t nseg,
                                                 const uint64_t* seg_begin, const uint32_t* seg_count,
                                                 const double* params, uint32_t n_params, uint32_t events_per_block,
                                                 double* sums) {
  if (!k || !in || !seg_begin || !seg_count || !sums || (n_params && !params))
    return fail(MF_ERR_INVALID, "null argument");
  const uint64_t chunk = events_per_block ? events_per_block : mfi::kMultiChunk;
  if (k->kind != MF_KERNEL_REDUCE) return fail(MF_ERR_INVALID, "kernel is not a REDUCE kernel");
  if (n_params != k->n_params) return fail(MF_ERR_INVALID, "parameter count mismatch");
  if (nseg == 0) return MF_OK;
  uint64_t end = 0;
  for (uint32_t s = 0; s < nseg; s++) end = std::max<uint64_t>(end, seg_begin[s] + seg_count[s]);
  int rc = check_layout(k, in, stride, end);
  if (rc) return rc;
  mf_context* c = k->ctx;
  MF_CUDA_TRY(cudaSetDevice(c->device));
  const void* data = nullptr;
  rc = prepare_input(k, in, stride, &data);
  if (rc) return rc;
  // a segment is a dataset that starts `begin` elements into every column
  const size_t eb = k->lowered.prep ? k->lowered.prep_elem_bytes() : elem_size(k->elem);
  std::vector<mfi::MultiItem> items;
  std::vector<uint32_t> where;  // item -> segment (empty segments have no item)
  items.reserve(nseg);
  for (uint32_t s = 0; s < nseg; s++) {
    if (seg_count[s] == 0) continue;
    items.push_back(mfi::MultiItem{k, static_cast<const char*>(data) + seg_begin[s] * eb, stride, seg_count[s],
                                   params + uint64_t(s) * n_params});
    where.push_back(s);
  }
  std::fill(sums, sums + size_t(nseg) * k->n_outputs, 0.0);
  if (items.empty()) return MF_OK;
  rc = ensure_scratch(c, 0, items.size() * k->n_outputs);
  if (rc) return rc;
  std::vector<unsigned char> host(mfi::multi_table_bytes(k, items, chunk));
  rc = mfi::launch_multi(c, k, items, host.data(), c->out_dev, chunk);
  if (rc) return rc;
  MF_CUDA_TRY(cudaStreamSynchronize(c->stream));
  for (size_t i = 0; i < items.size(); i++)
    std::memcpy(sums + size_t(where[i]) * k->n_outputs, c->out_host + i * k->n_outputs, k->n_outputs * sizeof(double));
  if (!k->desc) return MF_OK;
  // segments whose double-float sums are non-finite: again in native FP64
  std::vector<uint64_t> b2;
  std::vector<uint32_t> c2, bad;
  std::vector<double> p2;
  for (uint32_t s = 0; s < nseg; s++)
    if (!all_finite(sums + size_t(s) * k->n_outputs, k->n_outputs)) {
      bad.push_back(s);
      b2.push_back(seg_begin[s]);
      c2.push_back(seg_count[s]);
      p2.insert(p2.end(), params + uint64_t(s) * n_params, params + uint64_t(s + 1) * n_params);
    }
  if (bad.empty()) return MF_OK;
  rc = f64_twin(k);
  if (rc) return rc;
  k->fallbacks++;
  std::vector<double> s2(bad.size() * k->n_outputs);
  rc = mf_kernel_reduce_segments(k->f64, in, stride, uint32_t(bad.size()), b2.data(), c2.data(), p2.data(), n_params,
                                 s2.data());
  if (rc) return rc;
  for (size_t i = 0; i < bad.size(); i++)
    std::copy(s2.begin() + i * k->n_outputs, s2.begin() + (i + 1) * k->n_outputs, sums + size_t(bad[i]) * k->n_outputs);
  return MF_OK;
}
