// Debug build only (-DEFF_DEBUG): the bounds-checked variant of the library
// holds the frame-64 and frame-128 kernels, which every small parity fixture
// uses; the other frames and the persistent batch answer "unsupported".  In
// the product build this file compiles to nothing.
#ifdef EFF_DEBUG
#include "eff_internal.h"
#include "eff_launch.cuh"
#include "../../include/vmbd_eff.h"

namespace eff {
cudaError_t launch_n192(int, int, const Params&, int, int, int, size_t, cudaStream_t, const CUtensorMap*) {
  return cudaErrorNotSupported;
}
cudaError_t launch_n256(int, int, const Params&, int, int, int, size_t, cudaStream_t, const CUtensorMap*) {
  return cudaErrorNotSupported;
}
cudaError_t launch_n512(int, int, const Params&, int, int, int, size_t, cudaStream_t, const CUtensorMap*) {
  return cudaErrorNotSupported;
}
}  // namespace eff

extern "C" {
static int unsupported() { return eff::set_error(EFF_ERR_UNSUPPORTED, "not in the debug build"); }
int eff_batch_create(const EffPlan* const*, const int*, int, EffBatch**) { return unsupported(); }
int eff_batch_destroy(EffBatch*) { return EFF_OK; }
int eff_batch_items(const EffBatch*) { return 0; }
int eff_batch_forward_both(const EffBatch*, const float* const*, const float* const*, float* const*, void* const*,
                           void* const*, void*) {
  return unsupported();
}
int eff_batch_forward_residual(const EffBatch*, const float* const*, const float* const*, const float* const*,
                               float* const*, void* const*, void* const*, void*) {
  return unsupported();
}
int eff_batch_adjoint_residual(const EffBatch*, const float* const*, const float* const*, const void* const*,
                               const void* const*, float* const*, float* const*, double* const*, void*) {
  return unsupported();
}
}  // extern "C"
#endif  // EFF_DEBUG
