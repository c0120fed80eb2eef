// Total Lagrangian kernels, elementwise gradients and boundary loads.
#include "common.cuh"

int tl_material_tangent_impl(llf_ctx *ctx, llf_mesh *, llf_pattern *, const double *, int,
                             const double *, int, llf_matrix *) {
  return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "materialTangentMatrix: not built yet");
}
int tl_initial_stress_impl(llf_ctx *ctx, llf_mesh *, llf_pattern *, const double *,
                           const double *, int, const double *, int, llf_matrix *) {
  return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "initialStressMatrix: not built yet");
}
int tl_internal_force_impl(llf_ctx *ctx, llf_mesh *, const double *, const double *, int,
                           const double *, int, double *) {
  return llf_fail(ctx, LLF_ERR_UNSUPPORTED, "internalForceVector: not built yet");
}
