// Length-pass and sampling instantiations: planar B-splines of degree 4 and 5.
#include "gcv_length_hw.cuh"
#include "gcv_sample_impl.cuh"

namespace gcv {
GCV_LENGTH_INST2(0, bs_code(4, 2))
GCV_LENGTH_INST2(0, bs_code(5, 2))
GCV_SAMPLE_INST2(bs_code(4, 2))
GCV_SAMPLE_INST2(bs_code(5, 2))
GCV_LENGTH_HW_INST(bs_code(4, 2))
GCV_LENGTH_HW_INST(bs_code(5, 2))
}  // namespace gcv
