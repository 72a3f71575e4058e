/*
 * morefit_cuda.h — C ABI of the GB300 (sm_103a) likelihood backend for MoreFit.
 *
 * Plain C: opaque handles, pointers and sizes, int status codes, no CUDA or
 * C++ types in any signature. Every entry point returns MF_OK (0) or an
 * MF_ERR_* code and never aborts the process; mf_last_error() returns the
 * message of the calling thread's most recent failure.
 *
 * Each entry point below names the reference interface it replaces. The
 * reference's backend interface is the abstract C++ class
 * morefit::ComputeBlock<kernelT, evalT, seedT> (include/compute.hh:110-149)
 * plus ComputeBackend (include/compute.hh:98-107). include/compute_cuda.hh
 * implements those C++ classes on top of this ABI, so morefit::fitter,
 * generator and toystudy run unchanged on it.
 *
 * Data layout on the device: an event buffer is structure-of-arrays, column k
 * of a buffer with column stride S holds events [0, n) at element offset k*S
 * (the EventVector layout of include/eventvector.hh:236-260, with the stride
 * padded to a multiple of MF_COLUMN_ALIGN events so that every column starts
 * on a 256-byte boundary).
 */
#ifndef MOREFIT_CUDA_H
#define MOREFIT_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define MF_OK 0
#define MF_ERR_INVALID 1      /* bad argument (null handle, size, type, layout) */
#define MF_ERR_CUDA 2         /* a CUDA runtime call failed */
#define MF_ERR_NVRTC 3        /* runtime compilation of a generated kernel failed */
#define MF_ERR_PARSE 4        /* a kernel expression could not be parsed */
#define MF_ERR_BUDGET 5       /* allocation would exceed the context's HBM budget */
#define MF_ERR_NO_DEVICE 6    /* no CUDA device, or the device is not sm_103 */
#define MF_ERR_UNSUPPORTED 7  /* valid request this build does not implement */
#define MF_ERR_TIMEOUT 8      /* a bounded device wait gave up */
#define MF_ERR_NOT_READY 9    /* an asynchronous result is not ready yet (mf_coalesced_poll) */

/* ---- element types (kernelT of ComputeBlock<kernelT, evalT>) ---- */
#define MF_F64 0
#define MF_F32 1

/* ---- kernel kinds (how MakeComputeKernel's kahan flag and MakeGenerateKernel map) ---- */
#define MF_KERNEL_REDUCE 0    /* per-event values summed over events: MakeComputeKernel(kahan=true) */
#define MF_KERNEL_STORE 1     /* per-event values stored as output columns: MakeComputeKernel(kahan=false) */
#define MF_KERNEL_GENERATE 2  /* accept-reject event generation: MakeGenerateKernel */

#define MF_COLUMN_ALIGN 64    /* column stride granularity, events */
#define MF_MAX_PARAMS 512     /* parameter vector length limit per launch */
#define MF_MAX_OUTPUTS 512    /* outputs (graphs) per kernel */

typedef struct mf_context mf_context;
typedef struct mf_buffer mf_buffer;
typedef struct mf_kernel mf_kernel;
typedef struct mf_coalescer mf_coalescer;

/* Message of the calling thread's last failed call ("" if none). */
const char* mf_last_error(void);

/* Library version string. */
const char* mf_version(void);

/* Number of visible CUDA devices (0 without a GPU; never an error). */
int mf_device_count(int* count);

/* Name (NUL-terminated, at most len - 1 characters), SM count and compute
 * capability of device `device`; any output may be NULL. */
int mf_device_properties(int device, char* name, size_t len, int* sm_count, int* cc_major, int* cc_minor);

/* ---- context: one stream + scratch on one device ----
 * Replaces ComputeBackend construction (include/compute.hh:98-107; the
 * OpenCL backend's platform/device set-up, include/compute_opencl.hh:30-206).
 * hbm_budget_bytes caps the bytes of buffers allocated through this context
 * (0 = no cap). Calls on one context are serialised on its stream; use one
 * context per host thread for concurrency. */
int mf_context_create(int device, uint64_t hbm_budget_bytes, mf_context** out);
int mf_context_destroy(mf_context* ctx);
/* Bytes currently allocated through the context. */
int mf_context_allocated(const mf_context* ctx, uint64_t* bytes);
/* Blocks until all work queued on the context's stream has finished.
 * Replaces ComputeBlock::Finish (include/compute.hh:146). */
int mf_context_synchronize(mf_context* ctx);

/* ---- device buffers ----
 * Replace ComputeBlock::Setup{Input,Output,Parameter,Kahan,Seed}Buffer
 * (include/compute.hh:114-126). */
int mf_buffer_alloc(mf_context* ctx, uint64_t nbytes, mf_buffer** out);
int mf_buffer_free(mf_buffer* buf);
uint64_t mf_buffer_size(const mf_buffer* buf);
/* Raw device address (for interop); the buffer keeps ownership. Data written
 * through it is invisible to the prepared copies REDUCE kernels keep (see
 * mf_kernel_read_layout) until mf_buffer_mark_modified is called. */
void* mf_buffer_device_ptr(const mf_buffer* buf);
/* A buffer over caller-owned host memory that kernels read in place (the GPU
 * reads it over the host link while it computes; no copy to HBM): page-locked
 * memory is used through its mapped device address, other memory is
 * registered (mapped) until the buffer is freed. The memory must stay valid
 * while the buffer exists; mf_buffer_free releases the buffer, not the memory.
 * Counted in no HBM budget. For event blocks read once per step (the raw
 * events of a precompute kernel). */
int mf_buffer_wrap_host(mf_context* ctx, void* host, uint64_t nbytes, mf_buffer** out);
/* Declares that the buffer's contents changed outside the library (device
 * writes through mf_buffer_device_ptr, another library's kernels). Every
 * write made through this API (copies, memsets, uploads, STORE/GENERATE
 * outputs) does this by itself. No counterpart in the reference, whose
 * buffers are read as they are on every submit. */
int mf_buffer_mark_modified(mf_buffer* buf);
/* Plain byte copies (synchronous with respect to the host). */
int mf_buffer_h2d(mf_buffer* buf, uint64_t offset, const void* src, uint64_t nbytes);
int mf_buffer_d2h(const mf_buffer* buf, uint64_t offset, void* dst, uint64_t nbytes);
int mf_buffer_memset(mf_buffer* buf, int value);

/* Column stride (events) used on the device for n events: n rounded up to a
 * multiple of MF_COLUMN_ALIGN (at least MF_COLUMN_ALIGN). */
uint64_t mf_column_stride(uint64_t nevents);

/* Uploads an SoA event block with ncols columns of n events each, host
 * column stride host_stride (events), into buf with device column stride
 * dev_stride; the padding events of every column are zero-filled.
 * elem_type: MF_F64 or MF_F32 (the host data's type; no conversion).
 * Replaces ComputeBlock::CopyToInputBuffer (include/compute.hh:130). */
int mf_events_upload(mf_buffer* buf, int elem_type, const void* host, uint32_t ncols, uint64_t n,
                     uint64_t host_stride, uint64_t dev_stride);
/* Reverse of mf_events_upload. Replaces CopyFromOutputBuffer
 * (include/compute.hh:136). */
int mf_events_download(const mf_buffer* buf, int elem_type, void* host, uint32_t ncols, uint64_t n,
                       uint64_t host_stride, uint64_t dev_stride);
/* Uploads n FP64 values converting them to FP32 on the fly when elem_type is
 * MF_F32 (used to stage FP64 host events into an FP32 device layout). */
int mf_events_upload_f64_as(mf_buffer* buf, int elem_type, const double* host, uint32_t ncols, uint64_t n,
                            uint64_t host_stride, uint64_t dev_stride);
/* Stream-ordered forms of mf_events_upload and mf_buffer_d2h: enqueued on the
 * context's stream, they return at once. The host memory must stay valid and
 * unchanged (upload) or unread (download) until mf_context_synchronize; page-
 * locked host memory lets the copy overlap other work. With two contexts on
 * one device, one context's copies overlap the other's kernels (pipelined
 * evaluation of independent datasets). Split-phase form of the reference's
 * CopyToInputBuffer / CopyFromKahanBuffer (include/compute.hh:130-138), whose
 * OpenCL backend copies blocking (CL_TRUE, include/compute_opencl.hh:359,411). */
int mf_events_upload_async(mf_buffer* buf, int elem_type, const void* host, uint32_t ncols, uint64_t n,
                           uint64_t host_stride, uint64_t dev_stride);

/* Loads event columns from a file into buf (the on-disk input of the
 * reference, load_event_vector, include/eventvector.hh:297-332, reads a ROOT
 * TTree; this reads plain SoA files, e.g. the data of a 2-D .npy array):
 * at byte `offset` the file holds columns of file_stride values of file_elem
 * (MF_F64/MF_F32) each; file columns cols[0..ncols) become device columns
 * 0..ncols-1 (stride dev_stride, dev_elem), first n events of each, with the
 * padding events zero-filled; FP64 values stored as FP32 are rounded to
 * nearest. The file is read in 8 MiB chunks into two page-locked staging
 * buffers of the context, the read of one chunk overlapping the copy of the
 * other; returns once the data are on the device. A file shorter than the
 * columns it should hold is an MF_ERR_INVALID error. */
int mf_events_load_file(mf_buffer* buf, int dev_elem, uint64_t dev_stride, const char* path, uint64_t offset,
                        int file_elem, uint64_t file_stride, uint32_t ncols, const uint32_t* cols, uint64_t n);
int mf_buffer_d2h_async(const mf_buffer* buf, uint64_t offset, void* dst, uint64_t nbytes);

/* ---- kernels ----
 * Replaces ComputeBlock::MakeComputeKernel / MakeGenerateKernel
 * (include/compute.hh:140-144; the reference emits C/OpenCL text around
 * ComputeGraphNode::get_kernel() strings, include/compute_llvm.hh:535-750,
 * include/compute_opencl.hh:646-805). The expression strings are exactly
 * what get_kernel() prints (C syntax over input-column and parameter names,
 * constants as "%.15e" literals). The library parses them, shares common
 * subexpressions across all outputs, lowers them to CUDA C for the element
 * type, and compiles the kernel with NVRTC for sm_103a (cached by source). */
typedef struct mf_kernel_desc {
  const char* name;                 /* kernel name (diagnostics) */
  int kind;                         /* MF_KERNEL_REDUCE / STORE / GENERATE */
  int elem_type;                    /* MF_F64 or MF_F32: storage and arithmetic type */
  uint32_t n_inputs;                /* input column names, in buffer column order */
  const char* const* input_names;
  uint32_t n_params;                /* parameter names, in parameter-vector order */
  const char* const* param_names;
  uint32_t n_outputs;               /* one expression per output */
  const char* const* exprs;
  /* GENERATE only: n_outputs == 1 (the normalised density), the generated
   * dimensions are the n_gen_dims names below with ranges [lo, hi). */
  uint32_t n_gen_dims;
  const char* const* gen_dim_names;
  const double* gen_lo;
  const double* gen_hi;
  double maxprob;
  /* MF_FLAG_* bits. */
  uint32_t flags;
  /* Launch shape of REDUCE kernels (0 = library default): events per thread
   * per loop iteration (1, 2 or 4; vector loads of that width) and threads
   * per block (64..1024, multiple of 32). */
  uint32_t vec;
  uint32_t block;
  /* Shared-memory stages of the REDUCE input pipeline (0 = default, 2..8);
   * with direct loads, the unroll factor of the event loop (1..4). */
  uint32_t stages;
  /* Optional (NULL = none): for each of the n_params parameters, NULL or the
   * parameter-only expression that defines it in terms of the others, e.g.
   * the fitter's hoisted "morefit_parambuffer_k = (1-FS)*Fl"
   * (include/fitter.hh:381-396). Used only to find which input columns
   * always enter together when the lowering folds them; the parameter
   * vector passed at launch stays authoritative. */
  const char* const* param_defs;
} mf_kernel_desc;

/* FP64 REDUCE kernels evaluate the per-event expressions in double-float
 * arithmetic (pairs of FP32 values, ~48-bit significand, with FP64 sums) by
 * default, because GB300 issues FP32 at 64x its FP64 rate; this flag selects
 * native FP64 arithmetic instead. A double-float value has FP32's exponent
 * range (|x| up to 3.4e38): when mf_kernel_reduce or
 * mf_kernel_reduce_segments gets a non-finite sum from a double-float
 * kernel (an intermediate such as pow(x, n)^4 overflowed), it evaluates the
 * same launch (or the affected segments) again with a native-FP64 build of
 * the kernel, made on first need, and returns those sums
 * (mf_kernel_fallback_count counts such calls). The asynchronous and batched
 * entry points (mf_kernel_reduce_async, mf_kernel_reduce_many) return the
 * double-float sums as they are. Every REDUCE kernel, native FP64 included,
 * combines its per-thread partials across threads and blocks in
 * double-float, so the sums themselves must stay below 3.4e38 in magnitude
 * (likelihood, gradient and Hessian sums are many orders below). */
#define MF_FLAG_NATIVE_F64 1u
/* FP64 columns, FP32 per-event arithmetic with FP64 sums (the mixed-precision
 * form for raw observables that need their FP64 storage, e.g. a mass with a
 * large offset): a sum or difference of an input column and a parameter-only
 * value is formed in FP64 before rounding, everything else in FP32. */
#define MF_FLAG_F32_ARITH 2u
/* REDUCE kernels stream their input columns through a ring of shared-memory
 * stages filled by bulk asynchronous copies (cp.async.bulk + mbarrier, one
 * persistent block set) instead of the default grid-stride vector loads. */
#define MF_FLAG_BULK_PIPELINE 4u

int mf_kernel_build(mf_context* ctx, const mf_kernel_desc* desc, mf_kernel** out);
int mf_kernel_free(mf_kernel* k);
/* Copies the generated CUDA C source (NUL-terminated, truncated to len). */
int mf_kernel_source(const mf_kernel* k, char* buf, size_t len, size_t* needed);
/* Registers / spills / static shared memory reported by the compiler. */
int mf_kernel_info(const mf_kernel* k, int* regs, int* spill_bytes, int* block_size, int* vec_width);
/* What a kernel reads per event. A REDUCE kernel may read prepared columns
 * instead of its input buffer's: the lowering folds input columns that enter
 * every output only through the same parameter-weighted combinations (the
 * K*mumu P-wave's 11 hoisted angular columns fold to 9), and double-float
 * kernels read FP64 values pre-split into float pairs. The prepared copy is
 * made on the context's stream by the kernel's first launch on an input
 * buffer, kept beside that buffer (counted in the HBM budget, shared by the
 * kernels that prepare alike, freed with the buffer) and remade after the
 * buffer is written. columns / bytes_per_event: what the event loop reads;
 * source_columns: input columns the kernel uses. No counterpart in the
 * reference (its kernels read the hoisted columns as printed). */
int mf_kernel_read_layout(const mf_kernel* k, uint32_t* columns, uint32_t* bytes_per_event,
                          uint32_t* source_columns);

/* REDUCE: sums[j] = sum over events i in [0, n) of output j, accumulated
 * with per-thread partials, a warp/block tree and a compensated,
 * fixed-order combine of the block partials in the last block of the grid
 * (one launch, no host-side passes). FP64 kernels accumulate in FP64; FP32
 * kernels keep Kahan-compensated FP32 partials per thread and promote them
 * to FP64 at the warp level. Results are deterministic for a given n.
 * params: n_params FP64 values (converted to the element type on the device
 * side for FP32 kernels). input: column stride `stride` events; base and
 * stride must satisfy the MF_COLUMN_ALIGN layout. Synchronous: the last
 * block writes the sums to mapped host memory and then a completion word the
 * call spins on (a stream synchronize after 500 us, or on a launch error).
 * Replaces SubmitKernel + Finish + CopyFromKahanBuffer
 * (include/compute.hh:134-148, include/fitter.hh:1076-1096). */
int mf_kernel_reduce(mf_kernel* k, const mf_buffer* input, uint64_t stride, uint64_t n, const double* params,
                     uint32_t n_params, double* sums);

/* Enqueues one REDUCE launch on the context's stream and returns without
 * waiting; the n_outputs sums land in `out` at double offset
 * out_index * n_outputs once the stream reaches them. Launches on one
 * context run in stream order and share its scratch, so they never overlap
 * each other. Pair with mf_context_synchronize (Finish). */
int mf_kernel_reduce_async(mf_kernel* k, const mf_buffer* input, uint64_t stride, uint64_t n, const double* params,
                           uint32_t n_params, mf_buffer* out, uint64_t out_index);

/* Enqueues `count` REDUCE launches back to back on the context's stream
 * without host round trips: launch i reads inputs[i] (column stride
 * strides[i], ns[i] events) with parameter row i (params[i * n_params ...])
 * and writes its sums to row i of `out`. Used to evaluate many datasets or
 * parameter points per host call (several fits' requests, toy batches). */
int mf_kernel_reduce_many(mf_kernel* k, uint32_t count, const mf_buffer* const* inputs, const uint64_t* strides,
                          const uint64_t* ns, const double* params, uint32_t n_params, mf_buffer* out);

/* Evaluates `count` datasets (inputs[i], column stride strides[i], ns[i] >= 1
 * events, parameter row i) in ONE launch of the kernel's multi-dataset entry
 * plus one combine launch, enqueued on the context's stream; row i of `out`
 * receives dataset i's sums. Each dataset is cut into segments of 2048
 * events, one block per segment, and its segments' partial sums are combined
 * in a fixed order, so a dataset's sums are the same bit for bit whatever
 * else shares the launch (they differ from mf_kernel_reduce's, which sums in
 * another order, by rounding only). For many small datasets per host call,
 * where one launch per dataset (mf_kernel_reduce_many) is launch-bound:
 * concurrent fits, serving ticks. No counterpart in the reference, whose
 * blocks evaluate one dataset per SubmitKernel (compute.hh:146). */
int mf_kernel_reduce_multi(mf_kernel* k, uint32_t count, const mf_buffer* const* inputs, const uint64_t* strides,
                           const uint64_t* ns, const double* params, uint32_t n_params, mf_buffer* out);

/* ---- coalescing of concurrent host fitters ----
 * The reference runs one fitter per host thread, each calling
 * ComputeBlock::SubmitKernel + Finish + CopyFromKahanBuffer synchronously
 * from Minuit2's callbacks (minuit2_grad_fcn, fitter.hh:113-169;
 * likelihood_and_gradient, fitter.hh:1054-1151). A coalescer gathers the
 * synchronous evaluations that such threads make at about the same time and
 * runs them as shared launches (mf_kernel_reduce_multi's entry, one launch
 * pair per kernel source per tick) on its own stream, from one dispatch
 * thread.
 *
 * mf_coalescer_create starts the dispatch thread and a context of its own on
 * `device`. A tick starts when a request arrives and launches once every
 * attached context has a request waiting, `max_batch` requests are waiting
 * (0 = 256), or `window_us` microseconds have passed, whichever comes first.
 * mf_context_set_coalescer(ctx, co) routes every later mf_kernel_reduce on
 * ctx (the call CUDABlock::SubmitKernel makes) through co; NULL detaches.
 * The calling thread blocks until its tick completes, then returns the sums
 * as mf_kernel_reduce does (a double-float kernel's non-finite sums are
 * evaluated again in native FP64 on ctx, alone). A request's sums depend
 * only on its own data and parameters: the same alone or in any mix.
 * Detach every context before mf_coalescer_destroy (MF_ERR_INVALID
 * otherwise). Requests of one context must come from one thread at a time,
 * as the reference's blocks do. */
int mf_coalescer_create(int device, uint32_t max_batch, uint32_t window_us, mf_coalescer** out);
int mf_coalescer_destroy(mf_coalescer* co);
int mf_context_set_coalescer(mf_context* ctx, mf_coalescer* co);
/* Asynchronous form: submit returns a ticket at once (parameters copied);
 * poll with wait = 0 returns MF_ERR_NOT_READY until the tick has run, with
 * wait != 0 blocks; MF_OK writes the n_outputs sums and retires the ticket.
 * Sums are the tick's as launched (no native-FP64 re-evaluation). */
int mf_coalesced_submit(mf_coalescer* co, mf_kernel* k, const mf_buffer* input, uint64_t stride, uint64_t n,
                        const double* params, uint32_t n_params, uint64_t* ticket);
int mf_coalesced_poll(mf_coalescer* co, uint64_t ticket, double* sums, int wait);
/* Ticks run, evaluations served and the largest batch so far. */
int mf_coalescer_stats(const mf_coalescer* co, uint64_t* ticks, uint64_t* evaluations, uint32_t* max_batch);

/* ---- resident evaluations ----
 * With idle_us > 0, the synchronous mf_kernel_reduce calls of this context
 * (no coalescer attached) are watched; after a few calls the library builds,
 * in the background, a module with the REDUCE kernels used most (up to two
 * with the same block size, e.g. a fit's likelihood and likelihood+gradient)
 * and then serves their synchronous evaluations from one resident grid that
 * waits for requests in mapped host memory instead of launching a grid per
 * call. The sums are those of the kernel's own launch, bit for bit: each
 * request runs the kernel's own block partition and combine. The grid leaves
 * after idle_us without requests, or when any other work of this library is
 * launched on the device (by any context), and calls then launch as usual
 * until it is started again. Needs host-native atomics and cooperative
 * launches (MF_ERR_UNSUPPORTED otherwise). idle_us = 0 turns it off.
 * No counterpart in the reference (its backends launch per SubmitKernel). */
int mf_context_set_resident(mf_context* ctx, uint32_t idle_us);
/* state: -1 off, 0 watching calls, 1 building, 2 ready, 3 unavailable;
 * grids: resident grids launched; served: evaluations they served; blocks:
 * the resident grid's size (0 before it is built). */
int mf_context_resident_stats(const mf_context* ctx, int* state, uint64_t* grids, uint64_t* served, int* blocks);
/* The resident module for one or two REDUCE kernel descriptions, lowered and
 * compiled with NVRTC (no device needed): registers, spilled bytes and, when
 * source is non-NULL, its CUDA C (truncated to len). */
int mf_compile_check_resident(const mf_kernel_desc* const* descs, uint32_t count, int* regs, int* spill,
                              char* source, size_t len);


/* Compensated sums over events of ncols columns of an SoA event block:
 * sums[c] = sum_{i<n} column c (element type MF_F64 or MF_F32, column stride
 * `stride`), one launch, fixed summation order. Replaces the host-side
 * kahan_summation(EventVector, dim) (include/utils.hh:28-41) that the fitter
 * applies to per-event output buffers when kahan_on_accelerator is off
 * (include/fitter.hh:1082-1108), and the OpenCL backend's multi-pass Kahan
 * reduction kernels (include/compute_opencl.hh:807-991). */
int mf_columns_sum(const mf_buffer* buf, int elem_type, uint32_t ncols, uint64_t n, uint64_t stride, double* sums);

/* mf_columns_sum without any allocation. No counterpart in the reference:
 * it is for callers that cannot allocate device memory where they need the
 * sums -- code that hands out every device byte from its own arena or another
 * framework's allocator, a process whose allocation budget is spent, or a
 * latency-critical loop where cudaMalloc/cudaFree would synchronize the
 * device. It takes no context: `data` is a device pointer to ncols columns
 * (column stride `stride` elements, n events, element type MF_F64/MF_F32),
 * `sums` a device pointer to ncols doubles, `stream` a cudaStream_t (NULL for
 * the default stream). The call enqueues the work on that stream and
 * returns; the sums are valid once the stream has reached it. Results equal
 * mf_columns_sum's for the same data.
 *
 * Its scratch is a fixed 512 KiB + 256 B array in the library's device image
 * (held by every GPU that loads the library until the process exits): at
 * most 64 columns (MF_ERR_INVALID beyond that), any n. All calls on one GPU
 * share it and it keeps the last call's contents, so calls whose work
 * overlaps on the same GPU (two streams, two host threads) race and give
 * wrong sums: serialize them. Each GPU has its own copy. The first
 * call on a device looks up the array's device address on that device (a
 * one-time set-up); make that first call before any stream capture. That
 * address belongs to the device's primary context (the CUDA runtime's): do
 * not call the entry point from another driver context on the device, nor
 * after a cudaDeviceReset in the same process. The call allocates nothing
 * (no cudaMalloc/cudaFree, no allocating library routine); it clears its
 * completion counter with cudaMemsetAsync. */
int mf_columns_sum_noalloc(const void* data, int elem_type, uint32_t ncols, uint64_t n, uint64_t stride,
                           double* sums, void* stream);

/* Histogram of one event column for plotting (the data histogram of
 * plotter::plot, include/plotter.hh:296-319): event i goes to bin
 * floor((x_i - lo) / (hi - lo) * nbins), computed in FP64 as the reference
 * does. y[b] receives the number of events in bin b (weights == NULL) or the
 * sum of their weights, y2[b] the sum of squared weights (= y[b] without
 * weights). `data` and `weights` (NULL or the weight column) are device
 * pointers to n values of elem_type (MF_F64/MF_F32); y and y2 device pointers
 * to nbins doubles, `outside` a device pointer to one uint64 that receives
 * the number of events whose bin index is not in [0, nbins) (x >= hi, x < lo,
 * NaN) -- the reference throws for those. Unweighted counts are exact;
 * weighted sums are FP64 sums in an unspecified order. Enqueued on `stream`
 * (a cudaStream_t, NULL for the default stream); allocates nothing. */
int mf_histogram(const void* data, const void* weights, int elem_type, uint64_t n, double lo, double hi,
                 uint32_t nbins, double* y, double* y2, uint64_t* outside, void* stream);

/* The context's cudaStream_t, as an opaque pointer (interop: events, graphs). */
int mf_context_stream(mf_context* ctx, void** stream);

/* Ragged batched REDUCE over nseg independent event segments of one buffer
 * (toy studies): segment s covers events [seg_begin[s], seg_begin[s] +
 * seg_count[s]) of every column and uses parameter row s (params[s *
 * n_params ...]); sums[s * n_outputs + j]. One launch for all segments. */
int mf_kernel_reduce_segments(mf_kernel* k, const mf_buffer* input, uint64_t stride, uint32_t nseg,
                              const uint64_t* seg_begin, const uint32_t* seg_count, const double* params,
                              uint32_t n_params, double* sums);

/* mf_kernel_reduce_segments through the multi-dataset entry: each segment is
 * cut into runs of `events_per_block` events (0: 2048), one block each, whose
 * partial sums are combined in a fixed order, where mf_kernel_reduce_segments
 * gives each segment one block. A segment's sums depend on its own events,
 * parameters and the run length only. For segments long enough that one
 * block per segment leaves the device idle; the toy study's tuner picks the
 * entry and the run length. */
int mf_kernel_reduce_segments_chunked(mf_kernel* k, const mf_buffer* input, uint64_t stride, uint32_t nseg,
                                      const uint64_t* seg_begin, const uint32_t* seg_count, const double* params,
                                      uint32_t n_params, uint32_t events_per_block, double* sums);

/* How many mf_kernel_reduce / mf_kernel_reduce_segments calls on `k` were
 * evaluated again in native FP64 because a double-float sum was not finite
 * (see MF_FLAG_NATIVE_F64). */
int mf_kernel_fallback_count(const mf_kernel* k, uint64_t* count);

/* STORE: output column j of `output` (stride out_stride) receives output j
 * for events [0, n). Replaces SubmitKernel for non-Kahan and precompute
 * blocks (include/fitter.hh:345-375,704-712). */
int mf_kernel_store(mf_kernel* k, const mf_buffer* input, uint64_t in_stride, uint64_t n, const double* params,
                    uint32_t n_params, mf_buffer* output, uint64_t out_stride);
/* mf_kernel_store enqueued on the context's stream without waiting
 * (SubmitKernel without Finish). */
int mf_kernel_store_async(mf_kernel* k, const mf_buffer* input, uint64_t in_stride, uint64_t n, const double* params,
                          uint32_t n_params, mf_buffer* output, uint64_t out_stride);

/* GENERATE: accept-reject generation with one xoshiro128++ stream per
 * generator thread, as the reference's accelerator generate kernel
 * (include/compute_opencl.hh:425-645; seeds from include/generator.hh:115-135).
 * seeds: SoA [4][nseeds] host array; thread t produces events
 * [t*nper, min((t+1)*nper, n)) into output column d (stride out_stride) of
 * `out`. Every thread gives up after max_tries proposals (returns
 * MF_ERR_TIMEOUT) so a density that is never accepted cannot hang the GPU.
 * Replaces SubmitKernel + Finish of a generate block. */
int mf_kernel_generate(mf_kernel* k, const uint32_t* seeds, uint32_t nseeds, uint64_t n, uint64_t nper,
                       const double* params, uint32_t n_params, mf_buffer* out, uint64_t out_stride,
                       uint64_t max_tries);
/* mf_kernel_generate enqueued on the context's stream without waiting (the
 * seeds are copied before it returns). A thread that gives up sets the
 * context's error word, which the next synchronous REDUCE call on the context
 * reports as MF_ERR_TIMEOUT. For admitting many datasets without host round
 * trips (the serving loop). */
int mf_kernel_generate_async(mf_kernel* k, const uint32_t* seeds, uint32_t nseeds, uint64_t n, uint64_t nper,
                             const double* params, uint32_t n_params, mf_buffer* out, uint64_t out_stride,
                             uint64_t max_tries);
/* mf_kernel_generate_async with nstreams streams seeded on the device: stream
 * t starts from the state mf_splitmix_seed_rows(seed, nstreams) gives row t,
 * so the events equal those of that seed table, without building or copying
 * it (16 bytes per stream). For generations that need independent streams
 * rather than the reference's jump partition (e.g. a server generating each
 * request's dataset at admission). */
int mf_kernel_generate_splitmix_async(mf_kernel* k, uint64_t seed, uint32_t nstreams, uint64_t n, uint64_t nper,
                                      const double* params, uint32_t n_params, mf_buffer* out, uint64_t out_stride,
                                      uint64_t max_tries);

/* GENERATE for many datasets at once (toy studies with a different truth per
 * toy): segment s owns output events [seg_begin[s], seg_begin[s] +
 * seg_count[s]) and is generated by threads_per_seg xoshiro128++ streams
 * (seeds: SoA [4][nthreads], nthreads = nseg x threads_per_seg; stream r of
 * segment s fills the r-th block of ceil(count / threads_per_seg) events)
 * with parameter row s (seg_params[s * n_params ...]) and accept-reject bound
 * seg_maxprob[s]. The reference generates one toy per generator call
 * (include/toystudy.hh:62-75, include/generator.hh:71-175); this is the
 * batched form of the same accept-reject loop. */
int mf_kernel_generate_segments(mf_kernel* k, const uint32_t* seeds, uint32_t nthreads, uint32_t threads_per_seg,
                                uint32_t nseg, const uint64_t* seg_begin, const uint32_t* seg_count,
                                const double* seg_params, uint32_t n_params, const double* seg_maxprob,
                                mf_buffer* out, uint64_t out_stride, uint64_t max_tries);

/* Host evaluation of parameter-only expressions (the hoisted parameter
 * buffers "morefit_parambuffer_k" that the fitter evaluates before every
 * launch). Replaces ComputeGraphNode::eval (include/graph.hh:193) as used by
 * include/fitter.hh:1063-1072. out[i] = value of exprs[i]; an expression that
 * names a variable not in `names` is an MF_ERR_PARSE error. */
int mf_eval_expressions(uint32_t n_names, const char* const* names, const double* values, uint32_t n_exprs,
                        const char* const* exprs, double* out);
/* mf_eval_expressions for n_rows parameter vectors at once (values row-major
 * [n_rows][n_names], out [n_rows][n_exprs]); the expressions are parsed once.
 * The per-toy form of the same fitter step for batched toy fits
 * (include/toystudy.hh:55-82 runs one fitter per toy). */
int mf_eval_expressions_batch(uint32_t n_names, const char* const* names, uint32_t n_rows, const double* values,
                              uint32_t n_exprs, const char* const* exprs, double* out);
/* The same with the expressions parsed once into a handle, for callers that
 * evaluate them at every step (a fitter's per-evaluation parameter buffers,
 * a server's many concurrent fits): out [n_rows][n_exprs]. */
typedef struct mf_expr_set mf_expr_set;
int mf_expr_set_create(uint32_t n_names, const char* const* names, uint32_t n_exprs, const char* const* exprs,
                       mf_expr_set** out);
int mf_expr_set_eval(const mf_expr_set* set, uint32_t n_rows, const double* values, double* out);
int mf_expr_set_free(mf_expr_set* set);

/* Seed rows for the accelerator generator (include/generator.hh:115-135):
 * an xoshiro128++ state seeded like Xoshiro128pp::setSeed(seed)
 * (include/random.hh:355-362), row t = the state after t jump() calls
 * (include/random.hh:395-420). out is SoA [4][nrows]. */
int mf_seed_rows(uint64_t seed, uint32_t nrows, uint32_t* out);
/* Independent xoshiro128++ states for generations that need no reference
 * partition (toy datasets at their own truths, serving): row r = the upper
 * halves of four SplitMix64 outputs from (seed mod 2^32) * 2^32 + r.
 * out is SoA [4][nrows]. */
int mf_splitmix_seed_rows(uint64_t seed, uint32_t nrows, uint32_t* out);
/* Host linear algebra of batched fits (many small Newton systems; the
 * reference solves one fit at a time inside Minuit2): for each of n
 * symmetric p x p matrices H_t (row-major, back to back), Cholesky-factors
 * H_t and, where it is positive definite (ok[t] = 1), writes x_t = H_t^-1 g_t
 * (when g and x are given) and diag(H_t^-1) to dinv (when given). ok[t] = 0
 * leaves x_t and dinv_t unwritten. p <= 64. */
int mf_spd_solve_batch(uint32_t n, uint32_t p, const double* h, const double* g, double* x, double* dinv,
                       unsigned char* ok);

/* Work partition of the reference's accelerator generator for n events with
 * at most max_workitems generator threads (compute_opencl.hh:437-445,
 * generator.hh:120-128; max_workitems 8192 is compute_options' default):
 * *nper events per thread, *nseeds seed rows. */
int mf_generate_partition(uint64_t n, uint32_t max_workitems, uint64_t* nper, uint32_t* nseeds);

/* ---- diagnostics that need no GPU ----
 * Lowers a kernel description to CUDA C without compiling it. */
int mf_lower_source(const mf_kernel_desc* desc, char* buf, size_t len, size_t* needed);
/* Lowers and compiles (NVRTC, sm_103a) without loading: reports registers
 * and spill bytes per thread of the main entry. */
int mf_compile_check(const mf_kernel_desc* desc, int* regs, int* spill_bytes);

#ifdef __cplusplus
}
#endif
#endif /* MOREFIT_CUDA_H */
