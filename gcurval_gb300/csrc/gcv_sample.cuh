// Launcher of the sampling kernels (k_sample, FP64; k_sample_ff, mixed),
// defined in gcv_sample_impl.cuh and instantiated per curve code in the
// gcv_codes_*.cu units.
#pragma once

#include "gcv_kernels.cuh"

namespace gcv {

// PREC 0: k_sample<CODE>; PREC 1: k_sample_ff<CODE> on the float-float
// coefficients coef_ff.  CODE -1 dispatches per sample.
template <int CODE, int PREC>
cudaError_t sample_launch(const SampleParams& P, const float2* coef_ff, cudaStream_t stream, int grid, int threads);

}  // namespace gcv
