// Compile-time-length power-of-two passes, FP64 instances.
#include "passes_ct.cuh"

namespace bri17gb {
BRI17_CT_INSTANTIATE(double)

void ct_set_smem_attrs(size_t max_smem) {
  ct_set_smem_attrs_t<float>(max_smem);
  ct_set_smem_attrs_t<double>(max_smem);
  ct_set_smem_attrs_tma_f32(max_smem);
}
}  // namespace bri17gb
