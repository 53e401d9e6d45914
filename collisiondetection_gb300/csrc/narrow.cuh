// Launchers for the primitive narrow-phase kernels (narrow.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ccd {

// Device counters accumulated by the kernels of one batch.
struct BatchCounters {
  unsigned long long survivors;
  unsigned long long hits;
  unsigned long long status_flags;
  unsigned long long pad;
};

struct PrimBatch {
  int kind;
  int64_t n;
  const double *rows;  // n x width(kind) doubles
  const double *eta;   // 1 or n values
  int eta_per_row;
  uint8_t *hit;        // n
  double *t;           // n, written where hit
  uint8_t *status;     // n or nullptr
  BatchCounters *counters;
};

inline int row_width(int kind) { return kind <= 1 ? 24 : (kind == 2 ? 18 : 12); }

// FP64 evaluation of every row.
cudaError_t launch_prims_fp64(const PrimBatch &b, int num_sms, cudaStream_t s);

// FP32 conservative rejection (vertex-face, edge-edge, vertex-edge): rows that
// can be excluded get hit = 0; the others are appended to `survivors` (count
// in counters->survivors).
cudaError_t launch_prims_cull(const PrimBatch &b, int32_t *survivors, int num_sms, cudaStream_t s);
// Vertex-face and edge-edge survivors are refined by the staged kernels
// (stages.cuh); vertex-edge survivors by one FP64 pass over the list:
cudaError_t launch_prims_fp64_list(const PrimBatch &b, const int32_t *survivors, int num_sms, cudaStream_t s);

}  // namespace ccd
