// Pinned staging buffers and parallel host copies for streaming host sample
// arrays (gcv_staging.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>

namespace gcv {

constexpr int STAGE_SLOTS = 4;                 // two input, two output buffers
constexpr size_t STAGE_CHUNK = 256ull << 20;   // bytes of one chunk of positions

// memcpy split over a process-wide pool of host threads
void host_copy(void* dst, const void* src, size_t n);

// The staging buffers are shared by every context of the process: hold this
// lock while using them.
std::unique_lock<std::mutex> staging_lock();

// Pinned buffer i (0 .. STAGE_SLOTS-1) of at least `bytes`, grown on demand.
cudaError_t staging_slot(int i, size_t bytes, void** out);

}  // namespace gcv
