// Dispatch of the primitive narrow-phase launchers by kind.
#include "narrow.cuh"

namespace ccd {

cudaError_t launch_vf_fp64(const PrimBatch &, int, cudaStream_t);
cudaError_t launch_ee_fp64(const PrimBatch &, int, cudaStream_t);
cudaError_t launch_ve_fp64(const PrimBatch &, int, cudaStream_t);
cudaError_t launch_vv_fp64(const PrimBatch &, int, cudaStream_t);
cudaError_t launch_vf_cull(const PrimBatch &, int32_t *, int, cudaStream_t);
cudaError_t launch_ee_cull(const PrimBatch &, int32_t *, int, cudaStream_t);
cudaError_t launch_ve_cull(const PrimBatch &, int32_t *, int, cudaStream_t);
cudaError_t launch_ve_fp64_list(const PrimBatch &, const int32_t *, int, cudaStream_t);

cudaError_t launch_prims_fp64(const PrimBatch &b, int num_sms, cudaStream_t s) {
  if (b.n <= 0) return cudaSuccess;
  switch (b.kind) {
    case 0: return launch_vf_fp64(b, num_sms, s);
    case 1: return launch_ee_fp64(b, num_sms, s);
    case 2: return launch_ve_fp64(b, num_sms, s);
    default: return launch_vv_fp64(b, num_sms, s);
  }
}

cudaError_t launch_prims_cull(const PrimBatch &b, int32_t *list, int num_sms, cudaStream_t s) {
  if (b.n <= 0) return cudaSuccess;
  if (b.kind == 0) return launch_vf_cull(b, list, num_sms, s);
  if (b.kind == 1) return launch_ee_cull(b, list, num_sms, s);
  if (b.kind == 2) return launch_ve_cull(b, list, num_sms, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_prims_fp64_list(const PrimBatch &b, const int32_t *list, int num_sms, cudaStream_t s) {
  if (b.n <= 0) return cudaSuccess;
  if (b.kind == 2) return launch_ve_fp64_list(b, list, num_sms, s);
  return cudaErrorInvalidValue;
}

}  // namespace ccd
