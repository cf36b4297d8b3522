// jfem_apply_tet4.cu — element-kernel instantiations for Tet4.
#include "jfem_apply_kernels.cuh"

namespace jfem {
void launch_apply_tet4(Ctx* c, bool fp32, int mode, const double* v, const float2* v2, bool mask_in,
                        const int* stop) {
  launch_apply_et<JFEM_TET4>(c, fp32, mode, v, v2, mask_in, stop);
}
void launch_tile_tet4(Ctx* c, const float2* v2, float* y, bool masked, double* part, const int* stop) {
  launch_tile_et<JFEM_TET4>(c, v2, y, masked, part, stop);
}
void nh_state_tet4(Ctx* c) { nh_state_et<JFEM_TET4>(c); }
}  // namespace jfem
