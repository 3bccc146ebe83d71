// Length-pass and sampling instantiations: ellipses, and the runtime-dispatch deep passes.
#include "gcv_length_hw.cuh"
#include "gcv_sample_impl.cuh"

namespace gcv {
GCV_LENGTH_INST2(0, CODE_ELLIPSE)
GCV_LENGTH_INST2(1, CODE_ELLIPSE)
GCV_LENGTH_INST2(2, CODE_ELLIPSE)
GCV_LENGTH_INST2(1, -1)
GCV_LENGTH_INST2(2, -1)
GCV_SAMPLE_INST2(CODE_ELLIPSE)
GCV_LENGTH_HW_INST(CODE_ELLIPSE)
}  // namespace gcv
