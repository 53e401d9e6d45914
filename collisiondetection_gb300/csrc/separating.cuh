// SeparatingPlaneNarrowPhase on the device (separating.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ccd {

// A multi-entry History on the device: vertex v's entries are off[v] ..
// off[v+1]-1 of t (times) and p ([entries][3] positions).
struct HistoryView {
  const int32_t *off;
  const double *t, *p;
};

// SeparatingPlaneNarrowPhase::checkVFS (kind 0) / checkEES (kind 1) on n
// stencils (device [n][4], canonicalised here) with eps =
// History::computeMinimumGap() / 4: hit[i] 0/1; status[i] 1 where the
// interval search stalled (the reference overflows its stack there) and was
// stopped, hit then 0.
cudaError_t launch_separating_plane(int kind, const HistoryView &h, const int32_t *stencils, int64_t n,
                                    const double *eta, int eta_per_row, double eps, uint8_t *hit, uint8_t *status,
                                    cudaStream_t s);

// The two-entry history (start at time 0, end at time 1) of positions qs / qe
// as a HistoryView: off [nv + 1], t [2 nv], p [2 nv][3].
cudaError_t launch_two_entry_view(int nv, const double *qs, const double *qe, int32_t *off, double *t, double *p,
                                  cudaStream_t s);

}  // namespace ccd
