// Closest-point kernels of the reference's Distance class (include/Distance.h,
// src/Distance.cpp) on the device: primitive batches and the stencil stage of
// meshSelfDistance.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ccd {

// Row widths (doubles): vertex-face and vertex-plane rows are (p, q0, q1, q2),
// edge-edge and line-line rows (p0, p1, q0, q1); 12 doubles each.
constexpr int kDistanceRowWidth = 12;

// Distance::vertexFaceDistance (kind 0) / edgeEdgeDistance (kind 1) per row:
// vec [n][3] the returned vector; bary [n][3] / [n][4] the barycentric
// coordinates (may be null).
cudaError_t launch_distance_rows(int kind, int64_t n, const double *rows, double *vec, double *bary, int num_sms,
                                 cudaStream_t s);

// Distance::vertexPlaneDistanceLessThan (kind 0) / lineLineDistanceLessThan
// (kind 1) per row: out [n] 0/1; eta holds n values when eta_per_row, else 1.
cudaError_t launch_distance_less_than(int kind, int64_t n, const double *rows, const double *eta, bool eta_per_row,
                                      uint8_t *out, int num_sms, cudaStream_t s);

// The stencil stage of Distance::meshSelfDistance (src/Distance.cpp:49-64):
// lowers *best (device; the bits of a non-negative double, +inf to start) to
// the least |vertexFaceDistance(p, q0, q1, q2)| over the vertex-face stencils
// and |edgeEdgeDistance(p0, p1, q0, q1)| over the edge-edge stencils
// ([n][4] int32 on the device), positions x [nv][3].  NaN distances never
// lower it, as `dist < closest` in the reference.
cudaError_t launch_stencil_distance_min(const double *x, const int32_t *vf, int64_t n_vf, const int32_t *ee,
                                        int64_t n_ee, unsigned long long *best, int num_sms, cudaStream_t s);

}  // namespace ccd
