// Narrow-phase kernels for vertex-face rows (see narrow_kernels.cuh).
#include "narrow_kernels.cuh"

namespace ccd {

cudaError_t launch_vf_fp64(const PrimBatch &b, int num_sms, cudaStream_t s) {
  return kernels::fp64<kVF>(b, num_sms, s);
}
cudaError_t launch_vf_cull(const PrimBatch &b, int32_t *list, int num_sms, cudaStream_t s) {
  return kernels::cull<kVF>(b, list, num_sms, s);
}

}  // namespace ccd
