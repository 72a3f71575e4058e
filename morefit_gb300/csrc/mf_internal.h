// Declarations shared by the library's translation units (not part of the C ABI).
#ifndef MF_INTERNAL_H
#define MF_INTERNAL_H

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

// Records msg as the calling thread's last error and returns code.
int set_error(int code, const std::string& msg);

namespace mfi {
// Enqueues the column-sum kernel of mf_columns.cu: sums of ncols columns
// (element type elem, column stride `stride`, n events) into out[0..ncols),
// with `partials` holding columns_sum_partials(n, num_sms) * ncols float2 and
// `counter` a zeroed unsigned.
int columns_sum_launch(const void* data, int elem, uint64_t stride, uint64_t n, uint32_t ncols, void* partials,
                       unsigned* counter, double* out, cudaStream_t stream, int num_sms);
// Number of partial rows (blocks) the column-sum kernel uses for n events.
int columns_sum_partials(uint64_t n, int num_sms);
// Asks a resident evaluation grid on `device` (mf_context_set_resident), if
// one is up, to leave once idle, so that a launch that follows is not held
// back; no allocation, no synchronization.
void resident_yield_device(int device);
}  // namespace mfi

#endif
