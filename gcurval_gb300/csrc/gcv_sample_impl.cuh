// Definition of sample_launch (gcv_sample.cuh); included only by the
// gcv_codes_*.cu units that instantiate it.
#pragma once

#include "gcv_mixed.cuh"
#include "gcv_sample.cuh"

namespace gcv {

template <int CODE, int PREC>
cudaError_t sample_launch(const SampleParams& P, const float2* coef_ff, cudaStream_t stream, int grid, int threads)
{
    if constexpr (PREC == 1)
        k_sample_ff<CODE><<<grid, threads, 0, stream>>>(P, coef_ff);
    else
        k_sample<CODE><<<grid, threads, 0, stream>>>(P);
    return cudaGetLastError();
}

#define GCV_SAMPLE_INST2(CODE)                                                                     \
    template cudaError_t sample_launch<CODE, 0>(const SampleParams&, const float2*, cudaStream_t, int, int); \
    template cudaError_t sample_launch<CODE, 1>(const SampleParams&, const float2*, cudaStream_t, int, int);

}  // namespace gcv
