// jfem_apply_tet10.cu — Tet10: tiled FP32 apply instantiations, and the
// dispatch to the two-phase element passes (compiled in jfem_apply_tet10_f32.cu
// and jfem_apply_tet10_f64.cu, separate translation units for a parallel build).
#include "jfem_apply_kernels.cuh"

namespace jfem {
void launch_apply_tet10_f32(Ctx* c, const double* v, const float2* v2, bool mask_in, const int* stop);
void launch_apply_tet10_f64(Ctx* c, int mode, const double* v, bool mask_in, const int* stop);

void launch_apply_tet10(Ctx* c, bool fp32, int mode, const double* v, const float2* v2, bool mask_in,
                        const int* stop) {
  if (fp32) launch_apply_tet10_f32(c, v, v2, mask_in, stop);
  else launch_apply_tet10_f64(c, mode, v, mask_in, stop);
}
void launch_tile_tet10(Ctx* c, const float2* v2, float* y, bool masked, double* part, const int* stop) {
  launch_tile_et<JFEM_TET10>(c, v2, y, masked, part, stop);
}
void nh_state_tet10(Ctx* c) { nh_state_et<JFEM_TET10>(c); }
}  // namespace jfem
