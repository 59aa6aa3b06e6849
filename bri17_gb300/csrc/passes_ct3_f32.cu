// Compile-time-length passes for lengths 3 * 2^k (the twelve-element
// engine), FP32 instances.
#include "passes_ct.cuh"

namespace bri17gb {
BRI17_CT3_INSTANTIATE(float)
}  // namespace bri17gb
