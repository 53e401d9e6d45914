// Narrow-phase kernels for the degenerate vertex-edge and vertex-vertex rows
// (see narrow_kernels.cuh).
#include "narrow_kernels.cuh"

namespace ccd {

cudaError_t launch_ve_fp64(const PrimBatch &b, int num_sms, cudaStream_t s) {
  return kernels::fp64<kVE>(b, num_sms, s);
}
cudaError_t launch_ve_cull(const PrimBatch &b, int32_t *list, int num_sms, cudaStream_t s) {
  return kernels::cull<kVE>(b, list, num_sms, s);
}
cudaError_t launch_ve_fp64_list(const PrimBatch &b, const int32_t *list, int num_sms, cudaStream_t s) {
  return kernels::fp64_list<kVE>(b, list, num_sms, s);
}
cudaError_t launch_vv_fp64(const PrimBatch &b, int num_sms, cudaStream_t s) {
  return kernels::fp64<kVV>(b, num_sms, s);
}

}  // namespace ccd
