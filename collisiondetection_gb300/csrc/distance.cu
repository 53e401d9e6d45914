// Closest-point kernels (distance.cuh) and their C entry points
// (include/ccd_gb300.h: ccd_distance_batch*, ccd_distance_less_than_batch).
#include <math.h>

#include <algorithm>

#include "ccd_distance.h"
#include "context.cuh"
#include "distance.cuh"

namespace ccd {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ v3d ldx(const double *x, int v) { return ld3(x + 3 * (int64_t)v); }

template <int KIND>
__global__ void __launch_bounds__(kThreads) distance_rows(int64_t n, const double *rows, double *vec, double *bary) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double *r = rows + i * kDistanceRowWidth;
    const v3d a = ld3(r), b = ld3(r + 3), c = ld3(r + 6), d = ld3(r + 9);
    v3d out;
    if constexpr (KIND == 0) {
      double w[3];
      out = vertex_face_closest(a, b, c, d, w);
      if (bary)
        for (int k = 0; k < 3; k++) bary[3 * i + k] = w[k];
    } else {
      double w[4];
      out = edge_edge_closest(a, b, c, d, w);
      if (bary)
        for (int k = 0; k < 4; k++) bary[4 * i + k] = w[k];
    }
    vec[3 * i] = out.x;
    vec[3 * i + 1] = out.y;
    vec[3 * i + 2] = out.z;
  }
}

template <int KIND>
__global__ void __launch_bounds__(kThreads) distance_less_than(int64_t n, const double *rows, const double *eta,
                                                               bool eta_per_row, uint8_t *out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double *r = rows + i * kDistanceRowWidth;
    const double e = eta[eta_per_row ? i : 0];
    const v3d a = ld3(r), b = ld3(r + 3), c = ld3(r + 6), d = ld3(r + 9);
    bool less;
    if constexpr (KIND == 0)
      less = vertex_plane_distance_less_than(a, b, c, d, e);
    else
      less = line_line_distance_less_than(a, b, c, d, e);
    out[i] = less ? 1 : 0;
  }
}

__global__ void __launch_bounds__(kThreads) stencil_distance_min(const double *x, const int32_t *vf, int64_t n_vf,
                                                                 const int32_t *ee, int64_t n_ee,
                                                                 unsigned long long *best) {
  double local = INFINITY;
  const int64_t total = n_vf + n_ee;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    double d;
    if (i < n_vf) {
      const int4 st = reinterpret_cast<const int4 *>(vf)[i];
      double w[3];
      d = norm(vertex_face_closest(ldx(x, st.x), ldx(x, st.y), ldx(x, st.z), ldx(x, st.w), w));
    } else {
      const int4 st = reinterpret_cast<const int4 *>(ee)[i - n_vf];
      double w[4];
      d = norm(edge_edge_closest(ldx(x, st.x), ldx(x, st.y), ldx(x, st.z), ldx(x, st.w), w));
    }
    if (d < local) local = d;
  }
  unsigned long long b = (unsigned long long)__double_as_longlong(local);
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, b, o);
    b = other < b ? other : b;
  }
  if ((threadIdx.x & 31) == 0 && b < __ldcg(best)) atomicMin(best, b);
}

unsigned grid_for(int64_t n, int num_sms) {
  const int64_t blocks = (n + kThreads - 1) / kThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks, (int64_t)num_sms * 8));
}

}  // namespace

cudaError_t launch_distance_rows(int kind, int64_t n, const double *rows, double *vec, double *bary, int num_sms,
                                 cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (kind == 0)
    distance_rows<0><<<grid_for(n, num_sms), kThreads, 0, s>>>(n, rows, vec, bary);
  else
    distance_rows<1><<<grid_for(n, num_sms), kThreads, 0, s>>>(n, rows, vec, bary);
  return cudaGetLastError();
}

cudaError_t launch_distance_less_than(int kind, int64_t n, const double *rows, const double *eta, bool eta_per_row,
                                      uint8_t *out, int num_sms, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (kind == 0)
    distance_less_than<0><<<grid_for(n, num_sms), kThreads, 0, s>>>(n, rows, eta, eta_per_row, out);
  else
    distance_less_than<1><<<grid_for(n, num_sms), kThreads, 0, s>>>(n, rows, eta, eta_per_row, out);
  return cudaGetLastError();
}

cudaError_t launch_stencil_distance_min(const double *x, const int32_t *vf, int64_t n_vf, const int32_t *ee,
                                        int64_t n_ee, unsigned long long *best, int num_sms, cudaStream_t s) {
  if (n_vf + n_ee <= 0) return cudaSuccess;
  stencil_distance_min<<<grid_for(n_vf + n_ee, num_sms), kThreads, 0, s>>>(x, vf, n_vf, ee, n_ee, best);
  return cudaGetLastError();
}

}  // namespace ccd

// ------------------------------------------------------------------ C entry points
namespace {

using ccd_capi::fail;

// Rows per chunk of the host-memory entry points.
constexpr int64_t kDistanceChunk = 1 << 20;

int check_rows(ccd_context *ctx, int kind, int64_t n, const void *rows, const void *out) {
  if (!ctx) return CCD_ERR_INVALID_ARGUMENT;
  if (kind != 0 && kind != 1) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "unknown distance kind");
  if (n < 0 || n > INT32_MAX) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "n must be in [0, 2^31)");
  if (n > 0 && (!rows || !out)) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null buffer");
  return CCD_OK;
}

// Grows the context's distance scratch to `bytes`.
int ensure_dist(ccd_context *ctx, size_t bytes) {
  if (ctx->dist_cap >= bytes) return CCD_OK;
  CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  cudaFree(ctx->dist_mem);
  ctx->dist_mem = nullptr;
  ctx->dist_cap = 0;
  CCD_CUDA(cudaMalloc(&ctx->dist_mem, bytes));
  ctx->dist_cap = bytes;
  return CCD_OK;
}

}  // namespace

extern "C" {

int ccd_distance_batch_device(ccd_context *ctx, int kind, int64_t n, const double *rows, double *vec, double *bary) {
  int rc = check_rows(ctx, kind, n, rows, vec);
  if (rc || n == 0) return rc;
  CCD_CUDA(cudaSetDevice(ctx->device));
  CCD_CUDA(ccd::launch_distance_rows(kind, n, rows, vec, bary, ctx->num_sms, ctx->stream));
  return CCD_OK;
}

int ccd_distance_batch(ccd_context *ctx, int kind, int64_t n, const double *rows, double *vec, double *bary) {
  int rc = check_rows(ctx, kind, n, rows, vec);
  if (rc || n == 0) return rc;
  CCD_CUDA(cudaSetDevice(ctx->device));
  const int W = ccd::kDistanceRowWidth, B = kind == 0 ? 3 : 4;
  const int64_t chunk = std::min<int64_t>(n, kDistanceChunk);
  rc = ensure_dist(ctx, (size_t)chunk * (W + 3 + B) * sizeof(double));
  if (rc) return rc;
  double *d_rows = (double *)ctx->dist_mem, *d_vec = d_rows + chunk * W, *d_bary = d_vec + chunk * 3;
  for (int64_t off = 0; off < n; off += chunk) {
    const int64_t m = std::min(chunk, n - off);
    CCD_CUDA(cudaMemcpyAsync(d_rows, rows + off * W, (size_t)m * W * sizeof(double), cudaMemcpyHostToDevice,
                             ctx->stream));
    CCD_CUDA(ccd::launch_distance_rows(kind, m, d_rows, d_vec, bary ? d_bary : nullptr, ctx->num_sms, ctx->stream));
    CCD_CUDA(cudaMemcpyAsync(vec + off * 3, d_vec, (size_t)m * 3 * sizeof(double), cudaMemcpyDeviceToHost,
                             ctx->stream));
    if (bary)
      CCD_CUDA(cudaMemcpyAsync(bary + off * B, d_bary, (size_t)m * B * sizeof(double), cudaMemcpyDeviceToHost,
                               ctx->stream));
    CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return CCD_OK;
}

int ccd_distance_less_than_batch(ccd_context *ctx, int kind, int64_t n, const double *rows, const double *eta,
                                 int64_t eta_count, uint8_t *out) {
  int rc = check_rows(ctx, kind, n, rows, out);
  if (rc || n == 0) return rc;
  if (!eta || (eta_count != 1 && eta_count != n))
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "eta_count must be 1 or n");
  CCD_CUDA(cudaSetDevice(ctx->device));
  const int W = ccd::kDistanceRowWidth;
  const bool per_row = eta_count == n && n != 1;
  const int64_t chunk = std::min<int64_t>(n, kDistanceChunk);
  rc = ensure_dist(ctx, (size_t)chunk * (W + 1) * sizeof(double) + (size_t)chunk);
  if (rc) return rc;
  double *d_rows = (double *)ctx->dist_mem, *d_eta = d_rows + chunk * W;
  uint8_t *d_out = (uint8_t *)(d_eta + chunk);
  for (int64_t off = 0; off < n; off += chunk) {
    const int64_t m = std::min(chunk, n - off);
    CCD_CUDA(cudaMemcpyAsync(d_rows, rows + off * W, (size_t)m * W * sizeof(double), cudaMemcpyHostToDevice,
                             ctx->stream));
    CCD_CUDA(cudaMemcpyAsync(d_eta, per_row ? eta + off : eta, (size_t)(per_row ? m : 1) * sizeof(double),
                             cudaMemcpyHostToDevice, ctx->stream));
    CCD_CUDA(ccd::launch_distance_less_than(kind, m, d_rows, d_eta, per_row, d_out, ctx->num_sms, ctx->stream));
    CCD_CUDA(cudaMemcpyAsync(out + off, d_out, (size_t)m, cudaMemcpyDeviceToHost, ctx->stream));
    CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return CCD_OK;
}

}  // extern "C"
