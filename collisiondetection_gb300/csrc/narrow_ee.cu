// Narrow-phase kernels for edge-edge rows (see narrow_kernels.cuh).
#include "narrow_kernels.cuh"

namespace ccd {

cudaError_t launch_ee_fp64(const PrimBatch &b, int num_sms, cudaStream_t s) {
  return kernels::fp64<kEE>(b, num_sms, s);
}
cudaError_t launch_ee_cull(const PrimBatch &b, int32_t *list, int num_sms, cudaStream_t s) {
  return kernels::cull<kEE>(b, list, num_sms, s);
}

}  // namespace ccd
