// Length-pass and sampling instantiations: spatial B-splines of degree 1 to 3.
#include "gcv_length_hw.cuh"
#include "gcv_sample_impl.cuh"

namespace gcv {
GCV_LENGTH_INST2(0, bs_code(1, 3))
GCV_LENGTH_INST2(0, bs_code(2, 3))
GCV_LENGTH_INST2(0, bs_code(3, 3))
GCV_LENGTH_INST2(1, bs_code(3, 3))
GCV_LENGTH_INST2(2, bs_code(3, 3))
GCV_SAMPLE_INST2(bs_code(1, 3))
GCV_SAMPLE_INST2(bs_code(2, 3))
GCV_SAMPLE_INST2(bs_code(3, 3))
GCV_LENGTH_HW_INST(bs_code(1, 3))
GCV_LENGTH_HW_INST(bs_code(2, 3))
GCV_LENGTH_HW_INST(bs_code(3, 3))
}  // namespace gcv
