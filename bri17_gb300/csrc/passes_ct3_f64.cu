// Compile-time-length passes for lengths 3 * 2^k (the twelve-element
// engine), FP64 instances.
#include "passes_ct.cuh"

namespace bri17gb {
BRI17_CT3_INSTANTIATE(double)
}  // namespace bri17gb
