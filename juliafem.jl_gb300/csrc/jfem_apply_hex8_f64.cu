// jfem_apply_hex8_f64.cu — Hex8: FP64 element pass instantiations (K v / tangent, f_int).
#include "jfem_apply_kernels.cuh"

namespace jfem {
void launch_apply_hex8_f64(Ctx* c, int mode, const double* v, bool mask_in, const int* stop) {
  launch_apply_f64_et<JFEM_HEX8>(c, mode, v, mask_in, stop);
}
}  // namespace jfem
