// jfem_apply_hex8_f32.cu — Hex8: FP32 two-phase element pass instantiations.
#include "jfem_apply_kernels.cuh"

namespace jfem {
void launch_apply_hex8_f32(Ctx* c, const double* v, const float2* v2, bool mask_in, const int* stop) {
  launch_apply_f32_et<JFEM_HEX8>(c, v, v2, mask_in, stop);
}
}  // namespace jfem
