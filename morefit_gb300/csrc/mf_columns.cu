// Compensated sums of per-event columns on the device.
//
// Replaces the host-side Kahan summation of a block's per-event output
// buffer (reference include/utils.hh:28-41, used by include/fitter.hh:1082-1108
// when kahan_on_accelerator is off) and the OpenCL backend's separate
// multi-pass Kahan reduction kernels (include/compute_opencl.hh:807-991):
// one launch sums every column of an SoA block. Each thread keeps a
// double-float partial per column (FP32 pipe; GB300 issues FP64 at 1/64 of
// the FP32 rate), the block reduces them in a fixed order, every block
// writes its partials, and the last block to finish combines them in block
// order, so the result is reproducible for a given n.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/morefit_cuda.h"
#include "mf_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxGrid = 1024;  // partial rows per launch

struct dw {
  float h, l;
};
__device__ __forceinline__ dw two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ dw fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dw dw_add(dw a, dw b) {
  const dw s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, __fadd_rn(__fadd_rn(a.l, b.l), s.l));
}
// Exact-to-48-bits split of an FP64 value (one conversion; the column kernel
// is memory bound, so the FP64 pipe is not the limit here).
__device__ __forceinline__ dw split(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ dw split(float x) { return {x, 0.0f}; }
__device__ __forceinline__ dw shfl_xor(dw a, int o) {
  return {__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o)};
}

// One column at a time: grid-stride partial per thread, warp tree, block pass.
template <typename T>
__global__ void __launch_bounds__(kThreads) columns_sum_kernel(const T* __restrict__ data, uint64_t stride, uint64_t n,
                                                                uint32_t ncols, float2* __restrict__ partials,
                                                                unsigned* __restrict__ counter, double* __restrict__ out) {
  __shared__ float2 red[kThreads / 32];
  __shared__ bool am_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint32_t c = 0; c < ncols; c++) {
    const T* __restrict__ col = data + (uint64_t)c * stride;
    dw acc = {0.0f, 0.0f};
    for (uint64_t i = (uint64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kThreads)
      acc = dw_add(acc, split(col[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = dw_add(acc, shfl_xor(acc, o));
    if (lane == 0) red[warp] = make_float2(acc.h, acc.l);
    __syncthreads();
    if (threadIdx.x == 0) {
      dw b = {red[0].x, red[0].y};
      for (int w = 1; w < kThreads / 32; w++) b = dw_add(b, dw{red[w].x, red[w].y});
      partials[(uint64_t)blockIdx.x * ncols + c] = make_float2(b.h, b.l);
    }
    __syncthreads();
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  for (uint32_t c = 0; c < ncols; c++) {
    dw acc = {0.0f, 0.0f};
    for (unsigned b = threadIdx.x; b < gridDim.x; b += kThreads) {
      const float2 p = __ldcg(partials + (uint64_t)b * ncols + c);
      acc = dw_add(acc, dw{p.x, p.y});
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = dw_add(acc, shfl_xor(acc, o));
    if (lane == 0) red[warp] = make_float2(acc.h, acc.l);
    __syncthreads();
    if (threadIdx.x == 0) {
      dw b = {red[0].x, red[0].y};
      for (int w = 1; w < kThreads / 32; w++) b = dw_add(b, dw{red[w].x, red[w].y});
      out[c] = (double)b.h + (double)b.l;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *counter = 0u;
}

int grid_for(uint64_t n, int num_sms) {
  const uint64_t need = (n + kThreads - 1) / kThreads;
  const uint64_t cap = std::min<uint64_t>(kMaxGrid, uint64_t(num_sms) * 4);
  return int(std::max<uint64_t>(1, std::min(need, cap)));
}

}  // namespace

namespace mfi {

int columns_sum_launch(const void* data, int elem, uint64_t stride, uint64_t n, uint32_t ncols, void* partials,
                       unsigned* counter, double* out, cudaStream_t stream, int num_sms) {
  const int grid = grid_for(n, num_sms);
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) resident_yield_device(dev);
  if (elem == MF_F32)
    columns_sum_kernel<float><<<grid, kThreads, 0, stream>>>(static_cast<const float*>(data), stride, n, ncols,
                                                             static_cast<float2*>(partials), counter, out);
  else
    columns_sum_kernel<double><<<grid, kThreads, 0, stream>>>(static_cast<const double*>(data), stride, n, ncols,
                                                              static_cast<float2*>(partials), counter, out);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(MF_ERR_CUDA, std::string("columns_sum launch: ") + cudaGetErrorString(e));
  return MF_OK;
}

int columns_sum_partials(uint64_t n, int num_sms) { return grid_for(n, num_sms); }

}  // namespace mfi

// ---------------------------------------------------------------------------
// Column sums without any allocation.
//
// Some callers cannot allocate device memory at the point where they need
// these sums: code that hands every device byte out of its own arena or
// another framework's allocator, a process that has spent its allocation
// budget, or a latency-critical loop where cudaMalloc/cudaFree would
// synchronize the whole device. mf_columns_sum_noalloc serves them with the
// same kernel as mf_columns_sum, whose scratch (one partial row per block and
// a completion counter) lives in the file-scope arrays below instead of a
// context. Every GPU that loads this library holds these 512 KiB + 256 bytes
// until the process exits.
namespace {

constexpr uint32_t kNoAllocMaxCols = 64;  // largest ncols the entry point accepts
static __device__ __align__(256) float2 g_noalloc_partials[kMaxGrid * kNoAllocMaxCols];
static __device__ __align__(256) unsigned g_noalloc_counter;

constexpr int kMaxDevices = 64;
struct NoAllocScratch {
  bool ready = false;
  float2* partials = nullptr;  // device address of g_noalloc_partials on that device
  unsigned* counter = nullptr;
  int num_sms = 0;
};
NoAllocScratch g_noalloc[kMaxDevices];
std::mutex g_noalloc_mu;

// Once per device, with that device current: the device addresses of the
// scratch arrays (the names above are host-side stand-ins, not device
// addresses) and the SM count.
int noalloc_setup(int dev, NoAllocScratch** out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocScratch& s = g_noalloc[dev];
  if (!s.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess) return set_error(MF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    s.partials = static_cast<float2*>(p);
    e = cudaGetSymbolAddress(&p, g_noalloc_counter);
    if (e != cudaSuccess) return set_error(MF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    s.counter = static_cast<unsigned*>(p);
    e = cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return set_error(MF_ERR_CUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
    s.ready = true;
  }
  *out = &s;
  return MF_OK;
}

}  // namespace

extern "C" int mf_columns_sum_noalloc(const void* data, int elem_type, uint32_t ncols, uint64_t n, uint64_t stride,
                                      double* sums, void* stream) {
  if (!data || !sums) return set_error(MF_ERR_INVALID, "null argument");
  if (elem_type != MF_F64 && elem_type != MF_F32)
    return set_error(MF_ERR_INVALID, "element type must be MF_F64 or MF_F32");
  if (ncols == 0 || ncols > kNoAllocMaxCols)
    return set_error(MF_ERR_INVALID, "mf_columns_sum_noalloc: ncols must be 1.." + std::to_string(kNoAllocMaxCols) +
                                         " (its static scratch holds " + std::to_string(kNoAllocMaxCols) +
                                         " columns), got " + std::to_string(ncols));
  if (stride < n) return set_error(MF_ERR_INVALID, "column stride smaller than the number of events");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n == 0) {
    const cudaError_t e = cudaMemsetAsync(sums, 0, ncols * sizeof(double), st);
    if (e != cudaSuccess) return set_error(MF_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    return MF_OK;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(MF_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error(MF_ERR_INVALID, "device index beyond the supported range");
  NoAllocScratch* s = nullptr;
  int rc = noalloc_setup(dev, &s);
  if (rc) return rc;
  // The counter must start at zero; a previous call normally leaves it at
  // zero, clearing it on the caller's stream makes that unconditional.
  e = cudaMemsetAsync(s->counter, 0, sizeof(unsigned), st);
  if (e != cudaSuccess) return set_error(MF_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  return mfi::columns_sum_launch(data, elem_type, stride, n, ncols, s->partials, s->counter, sums, st, s->num_sms);
}

// ---- histogram of one column (plotting) ----
//
// Bin index as the reference's plotter computes it (plotter.hh:301-319):
// floor((x - lo) / (hi - lo) * nbins) in FP64, so every event lands in the
// same bin. Per-block shared-memory histograms (atomics) flushed to global
// memory; unweighted counts are integers (exact), accumulated in place in
// the output array's 8-byte words and converted to FP64 at the end.
namespace {

constexpr uint32_t kHistSharedCount = 8192;  // u32 counters in shared memory
constexpr uint32_t kHistSharedWeight = 2048;  // (sum w, sum w^2) pairs in shared memory

template <typename T, bool Weighted, bool Shared>
__global__ void __launch_bounds__(kThreads) histogram_kernel(const T* __restrict__ x, const T* __restrict__ w,
                                                              uint64_t n, double lo, double width, uint32_t nbins,
                                                              double* __restrict__ y, double* __restrict__ y2,
                                                              unsigned long long* __restrict__ outside) {
  extern __shared__ __align__(16) unsigned char hist_smem[];
  unsigned* scount = reinterpret_cast<unsigned*>(hist_smem);
  double* sw = reinterpret_cast<double*>(hist_smem);
  unsigned long long* gcount = reinterpret_cast<unsigned long long*>(y);
  if (Shared) {
    for (uint32_t b = threadIdx.x; b < nbins; b += blockDim.x) {
      if (Weighted) {
        sw[2 * b] = 0.0;
        sw[2 * b + 1] = 0.0;
      } else {
        scount[b] = 0u;
      }
    }
    __syncthreads();
  }
  const double nb = double(nbins);
  unsigned long long out = 0;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x) {
    const double f = floor((double(x[i]) - lo) / width * nb);
    if (!(f >= 0.0 && f < nb)) {
      out++;
      continue;
    }
    const uint32_t b = uint32_t(f);
    if (Weighted) {
      const double wi = double(w[i]);
      if (Shared) {
        atomicAdd(&sw[2 * b], wi);
        atomicAdd(&sw[2 * b + 1], wi * wi);
      } else {
        atomicAdd(&y[b], wi);
        atomicAdd(&y2[b], wi * wi);
      }
    } else {
      if (Shared)
        atomicAdd(&scount[b], 1u);
      else
        atomicAdd(&gcount[b], 1ull);
    }
  }
  if (out) atomicAdd(outside, out);
  if (Shared) {
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < nbins; b += blockDim.x) {
      if (Weighted) {
        if (sw[2 * b] != 0.0 || sw[2 * b + 1] != 0.0) {
          atomicAdd(&y[b], sw[2 * b]);
          atomicAdd(&y2[b], sw[2 * b + 1]);
        }
      } else if (scount[b]) {
        atomicAdd(&gcount[b], (unsigned long long)scount[b]);
      }
    }
  }
}

// Unweighted: integer counts (in y's words) to FP64 counts in y and y2.
__global__ void histogram_counts_to_f64(double* __restrict__ y, double* __restrict__ y2, uint32_t nbins) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbins) return;
  const double c = double(reinterpret_cast<const unsigned long long*>(y)[b]);
  y[b] = c;
  y2[b] = c;
}

template <typename T>
int histogram_launch(const void* data, const void* weights, uint64_t n, double lo, double width, uint32_t nbins,
                     double* y, double* y2, unsigned long long* outside, cudaStream_t st, int grid) {
  const T* x = static_cast<const T*>(data);
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) mfi::resident_yield_device(dev);
  const T* w = static_cast<const T*>(weights);
  if (w) {
    if (nbins <= kHistSharedWeight)
      histogram_kernel<T, true, true><<<grid, kThreads, size_t(nbins) * 16, st>>>(x, w, n, lo, width, nbins, y, y2,
                                                                                   outside);
    else
      histogram_kernel<T, true, false><<<grid, kThreads, 0, st>>>(x, w, n, lo, width, nbins, y, y2, outside);
  } else {
    if (nbins <= kHistSharedCount)
      histogram_kernel<T, false, true><<<grid, kThreads, size_t(nbins) * 4, st>>>(x, w, n, lo, width, nbins, y, y2,
                                                                                   outside);
    else
      histogram_kernel<T, false, false><<<grid, kThreads, 0, st>>>(x, w, n, lo, width, nbins, y, y2, outside);
    histogram_counts_to_f64<<<(nbins + kThreads - 1) / kThreads, kThreads, 0, st>>>(y, y2, nbins);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(MF_ERR_CUDA, std::string("histogram launch: ") + cudaGetErrorString(e));
  return MF_OK;
}

}  // namespace

extern "C" int mf_histogram(const void* data, const void* weights, int elem_type, uint64_t n, double lo, double hi,
                            uint32_t nbins, double* y, double* y2, uint64_t* outside, void* stream) {
  if (!data || !y || !y2 || !outside) return set_error(MF_ERR_INVALID, "null argument");
  if (elem_type != MF_F64 && elem_type != MF_F32)
    return set_error(MF_ERR_INVALID, "element type must be MF_F64 or MF_F32");
  if (nbins == 0) return set_error(MF_ERR_INVALID, "nbins must be positive");
  if (!(hi > lo)) return set_error(MF_ERR_INVALID, "histogram range must have hi > lo");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(y, 0, size_t(nbins) * sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(y2, 0, size_t(nbins) * sizeof(double), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(outside, 0, sizeof(uint64_t), st);
  if (e != cudaSuccess) return set_error(MF_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
  int dev = 0, sms = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return set_error(MF_ERR_CUDA, std::string("device query: ") + cudaGetErrorString(e));
  const uint64_t need = (n + uint64_t(kThreads) * 8 - 1) / (uint64_t(kThreads) * 8);
  const int grid = int(std::max<uint64_t>(1, std::min<uint64_t>(need, uint64_t(sms) * 4)));
  auto* outp = reinterpret_cast<unsigned long long*>(outside);
  const double width = hi - lo;
  return elem_type == MF_F64
             ? histogram_launch<double>(data, weights, n, lo, width, nbins, y, y2, outp, st, grid)
             : histogram_launch<float>(data, weights, n, lo, width, nbins, y, y2, outp, st, grid);
}
