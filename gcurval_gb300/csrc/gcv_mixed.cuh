// Mixed-precision path (FP32 integrand and panels; FP64 prefix sum, error
// test near tolerance and final Newton step).
#pragma once

#include "gcurval_gb300.h"
#include "gcv_kernels.cuh"

namespace gcv {
namespace mixed {

struct MixedState {
    int unused = 0;
};

inline void release(MixedState&) {}

inline gcv_status build_table(MixedState&, cudaStream_t, const Batch&, const Table&, int, double, int, int, cudaEvent_t*,
                              gcv_stats*, unsigned long long*, int64_t)
{
    return GCV_ERR_INVALID;
}

inline gcv_status sample(MixedState&, cudaStream_t, const Batch&, const Table&, const int64_t*, const double*, int64_t,
                         int, int, int, double*, int)
{
    return GCV_ERR_INVALID;
}

}  // namespace mixed
}  // namespace gcv
