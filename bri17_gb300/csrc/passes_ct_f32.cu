// Compile-time-length power-of-two passes, FP32 instances.
#include "passes_ct.cuh"

namespace bri17gb {
BRI17_CT_INSTANTIATE(float)
}  // namespace bri17gb
