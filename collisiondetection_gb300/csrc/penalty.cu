// Penalty forces of one group (include/ccd_gb300.h: ccd_penalty_group_force):
// PenaltyGroup::addForce (src/PenaltyGroup.cpp:34-52) with the potentials of
// VertexFacePenaltyPotential / EdgeEdgePenaltyPotential::addForce
// (src/PenaltyPotential.cpp:7-64).
//
// The reference adds each stencil's force into a zeroed group vector in
// stencil order (vertex-face stencils, then edge-edge ones; within a stencil
// p, q0, q1, q2), then F += group * dt.  Floating-point sums depend on their
// order, so the device keeps it: every stencil's contributions are computed in
// parallel, tagged (vertex, stencil sequence, slot), sorted by that tag, and
// each vertex's run is summed by one thread in tag order -- the reference's
// order -- starting from 0.0.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "context.cuh"
#include "penalty.cuh"
#include "radix_sort.cuh"

namespace ccd {

namespace {

constexpr int kThreads = 256;
constexpr int kSlotBits = 2;   // four contributions per stencil
constexpr int kSeqBits = 32;   // stencil sequence numbers below 2^30, tags below 2^32
constexpr int kTagBits = kSeqBits;

// Per stencil (sequence number base + i): fired flag, the four contribution
// vectors, and one tag per contribution, vertex << 32 | sequence << 2 | slot,
// appended at *ntags.
template <int KIND>
__global__ void __launch_bounds__(kThreads) penalty_stencils(const double *q, const double *vel, int nverts,
                                                             const int32_t *st, const uint8_t *isnew, int64_t n,
                                                             int64_t base, PenaltyParams pp, uint8_t *fired,
                                                             double *contrib, uint64_t *tags,
                                                             unsigned long long *ntags, unsigned int *newused,
                                                             unsigned int *bad) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  bool f = false;
  int v[4] = {0, 0, 0, 0};
  if (i < n) {
    v[0] = st[4 * i], v[1] = st[4 * i + 1], v[2] = st[4 * i + 2], v[3] = st[4 * i + 3];
    canonical(KIND, v);
    v3d c[4];
    const bool inside = (unsigned)v[0] < (unsigned)nverts && (unsigned)v[1] < (unsigned)nverts &&
                        (unsigned)v[2] < (unsigned)nverts && (unsigned)v[3] < (unsigned)nverts;
    if (!inside) atomicOr(bad, 1u);  // reported as an error; the stencil is skipped
    f = inside && stencil_force<KIND>(q, vel, v, pp, c);
    fired[i] = f ? 1 : 0;
    if (f) {
      double *out = contrib + 12 * (base + i);
      for (int k = 0; k < 4; k++) {
        out[3 * k] = c[k].x;
        out[3 * k + 1] = c[k].y;
        out[3 * k + 2] = c[k].z;
      }
      if (isnew && isnew[i]) atomicOr(newused, 1u);
    }
  }
  // Warp-aggregated append of four tags per fired stencil.
  const unsigned mask = __ballot_sync(0xffffffffu, f);
  if (!mask) return;
  const int lane = threadIdx.x & 31;
  unsigned long long first = 0;
  if (lane == __ffs(mask) - 1) first = atomicAdd(ntags, 4ull * __popc(mask));
  first = __shfl_sync(0xffffffffu, first, __ffs(mask) - 1);
  if (f) {
    const unsigned long long at = first + 4ull * __popc(mask & ((1u << lane) - 1));
    const uint64_t seq = (uint64_t)(base + i);
    for (int k = 0; k < 4; k++)
      tags[at + k] = ((uint64_t)(uint32_t)v[k] << kTagBits) | (seq << kSlotBits) | (uint64_t)k;
  }
}

// One thread per run of equal vertices in the sorted tags: the group force of
// that vertex, summed in tag order from 0.0 (src/PenaltyGroup.cpp:36-50 with
// the += / -= of src/PenaltyPotential.cpp:29-32, 59-62).
__global__ void __launch_bounds__(kThreads) penalty_sum(const uint64_t *tags, int64_t ntags, int64_t n_vf,
                                                        const double *contrib, double *group) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= ntags) return;
  const uint64_t vtx = tags[i] >> kTagBits;
  if (i > 0 && (tags[i - 1] >> kTagBits) == vtx) return;
  double gx = 0.0, gy = 0.0, gz = 0.0;
  for (int64_t j = i; j < ntags && (tags[j] >> kTagBits) == vtx; j++) {
    const uint64_t tag = tags[j] & 0xffffffffull;
    const int64_t seq = (int64_t)(tag >> kSlotBits);
    const int slot = (int)(tag & 3);
    const double *c = contrib + 12 * seq + 3 * slot;
    const bool minus = seq < n_vf ? slot == 0 : slot <= 1;
    if (minus) {
      gx = gx - c[0];
      gy = gy - c[1];
      gz = gz - c[2];
    } else {
      gx = gx + c[0];
      gy = gy + c[1];
      gz = gz + c[2];
    }
  }
  group[3 * vtx] = gx;
  group[3 * vtx + 1] = gy;
  group[3 * vtx + 2] = gz;
}

// F += group * dt (src/PenaltyGroup.cpp:50), every coordinate.
__global__ void __launch_bounds__(kThreads) penalty_apply(int64_t n3, const double *group, double dt, double *F) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n3) F[i] = F[i] + group[i] * dt;
}

unsigned grid_of(int64_t n) { return (unsigned)std::max<int64_t>(1, (n + kThreads - 1) / kThreads); }

}  // namespace

}  // namespace ccd

// ------------------------------------------------------------------ C entry points
namespace {

using ccd_capi::fail;

int check_args(ccd_context *ctx, int32_t nverts, const void *q, const void *v, const void *F, int64_t n_vf,
               const void *vf, int64_t n_ee, const void *ee) {
  if (!ctx) return CCD_ERR_INVALID_ARGUMENT;
  if (nverts < 0 || n_vf < 0 || n_ee < 0 || (nverts > 0 && (!q || !v || !F)) || (n_vf > 0 && !vf) ||
      (n_ee > 0 && !ee))
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null buffer or negative size");
  if (n_vf + n_ee >= ((int64_t)1 << 30)) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "2^30 or more stencils");
  return CCD_OK;
}

// The forces of one group from device buffers: vf and ee stencils in one
// array (vf first), isnew likewise (or null); F updated in place.
int penalty_device(ccd_context *ctx, int32_t nverts, const double *d_q, const double *d_v, int64_t n_vf, int64_t n_ee,
                   const int32_t *d_st, const uint8_t *d_new, const ccd::PenaltyParams &pp, double dt, double *d_F,
                   uint8_t *d_fired, int *newused) {
  cudaStream_t s = ctx->stream;
  const int64_t n = n_vf + n_ee, V3 = 3 * (int64_t)nverts;
  const int64_t ntag_cap = std::max<int64_t>(4 * n, 1);
  const size_t sort_temp = ccd::radix_sort_temp_bytes(ntag_cap);
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    const size_t at = off;
    off += (bytes + 255) / 256 * 256;
    return at;
  };
  const size_t o_g = carve(V3 * 8), o_c = carve((size_t)12 * std::max<int64_t>(n, 1) * 8);
  const size_t o_t = carve((size_t)ntag_cap * 8), o_t2 = carve((size_t)ntag_cap * 8), o_tmp = carve(sort_temp);
  const size_t o_cnt = carve(16);
  char *mem = nullptr;
  CCD_CUDA(cudaMallocAsync((void **)&mem, off, s));
  double *d_g = (double *)(mem + o_g), *d_c = (double *)(mem + o_c);
  uint64_t *d_t = (uint64_t *)(mem + o_t), *d_t2 = (uint64_t *)(mem + o_t2);
  unsigned long long *d_cnt = (unsigned long long *)(mem + o_cnt);
  auto run = [&]() -> int {
    CCD_CUDA(cudaMemsetAsync(d_g, 0, V3 * 8, s));
    CCD_CUDA(cudaMemsetAsync(d_cnt, 0, 16, s));
    unsigned int *d_newused = (unsigned int *)(d_cnt + 1), *d_bad = d_newused + 1;
    if (n_vf)
      ccd::penalty_stencils<0><<<ccd::grid_of(n_vf), ccd::kThreads, 0, s>>>(
          d_q, d_v, nverts, d_st, d_new, n_vf, 0, pp, d_fired, d_c, d_t, d_cnt, d_newused, d_bad);
    if (n_ee)
      ccd::penalty_stencils<1><<<ccd::grid_of(n_ee), ccd::kThreads, 0, s>>>(
          d_q, d_v, nverts, d_st + 4 * n_vf, d_new ? d_new + n_vf : nullptr, n_ee, n_vf, pp, d_fired + n_vf, d_c,
          d_t, d_cnt, d_newused, d_bad);
    CCD_CUDA(cudaGetLastError());
    unsigned long long hcnt[2] = {0, 0};
    CCD_CUDA(cudaMemcpyAsync(hcnt, d_cnt, 16, cudaMemcpyDeviceToHost, s));
    CCD_CUDA(cudaStreamSynchronize(s));
    if (hcnt[1] >> 32) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "stencil vertex out of range");
    const int64_t ntags = (int64_t)hcnt[0];
    if (ntags) {
      int vbits = 1;
      while (vbits < 31 && ((int64_t)1 << vbits) < nverts) vbits++;
      CCD_CUDA(ccd::radix_sort_u64(d_t, d_t2, nullptr, nullptr, ntags, 0, ccd::kTagBits + vbits, mem + o_tmp,
                                   sort_temp, s));
      ccd::penalty_sum<<<ccd::grid_of(ntags), ccd::kThreads, 0, s>>>(d_t, ntags, n_vf, d_c, d_g);
      CCD_CUDA(cudaGetLastError());
    }
    ccd::penalty_apply<<<ccd::grid_of(V3), ccd::kThreads, 0, s>>>(V3, d_g, dt, d_F);
    CCD_CUDA(cudaGetLastError());
    if (newused) *newused = (hcnt[1] & 0xffffffffull) ? 1 : 0;
    return CCD_OK;
  };
  const int rc = run();
  cudaFreeAsync(mem, s);
  return rc;
}

}  // namespace

extern "C" {

int ccd_penalty_group_force_device(ccd_context *ctx, int32_t nverts, const double *q, const double *v, int64_t n_vf,
                                   const int32_t *vf, const uint8_t *vf_isnew, int64_t n_ee, const int32_t *ee,
                                   const uint8_t *ee_isnew, double outer_eta, double inner_eta, double stiffness,
                                   double cor, double dt, double *F, uint8_t *vf_fired, uint8_t *ee_fired,
                                   int *newused) {
  int rc = check_args(ctx, nverts, q, v, F, n_vf, vf, n_ee, ee);
  if (rc) return rc;
  if (newused) *newused = 0;
  if (nverts == 0) return CCD_OK;
  if ((n_vf && !vf_fired) || (n_ee && !ee_fired))
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "the device entry point needs the fired arrays");
  CCD_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const int64_t n = n_vf + n_ee;
  // The kernels take the two stencil lists (and flags) as one array.
  int32_t *st = nullptr;
  uint8_t *nw = nullptr, *fired = nullptr;
  const size_t b_st = (size_t)16 * std::max<int64_t>(n, 1), b_n = (size_t)std::max<int64_t>(n, 1);
  CCD_CUDA(cudaMallocAsync((void **)&st, b_st + 2 * b_n + 512, s));
  nw = (uint8_t *)st + (b_st + 255) / 256 * 256;
  fired = nw + (b_n + 255) / 256 * 256;
  auto run = [&]() -> int {
    if (n_vf) CCD_CUDA(cudaMemcpyAsync(st, vf, (size_t)n_vf * 16, cudaMemcpyDeviceToDevice, s));
    if (n_ee) CCD_CUDA(cudaMemcpyAsync(st + 4 * n_vf, ee, (size_t)n_ee * 16, cudaMemcpyDeviceToDevice, s));
    CCD_CUDA(cudaMemsetAsync(nw, 0, b_n, s));
    if (n_vf && vf_isnew) CCD_CUDA(cudaMemcpyAsync(nw, vf_isnew, (size_t)n_vf, cudaMemcpyDeviceToDevice, s));
    if (n_ee && ee_isnew) CCD_CUDA(cudaMemcpyAsync(nw + n_vf, ee_isnew, (size_t)n_ee, cudaMemcpyDeviceToDevice, s));
    const ccd::PenaltyParams pp{outer_eta, inner_eta, stiffness, cor};
    const int r = penalty_device(ctx, nverts, q, v, n_vf, n_ee, st, nw, pp, dt, F, fired, newused);
    if (r) return r;
    if (n_vf) CCD_CUDA(cudaMemcpyAsync(vf_fired, fired, (size_t)n_vf, cudaMemcpyDeviceToDevice, s));
    if (n_ee) CCD_CUDA(cudaMemcpyAsync(ee_fired, fired + n_vf, (size_t)n_ee, cudaMemcpyDeviceToDevice, s));
    return CCD_OK;
  };
  rc = run();
  cudaFreeAsync(st, s);
  return rc;
}

int ccd_penalty_group_force(ccd_context *ctx, int32_t nverts, const double *q, const double *v, int64_t n_vf,
                            const int32_t *vf, const uint8_t *vf_isnew, int64_t n_ee, const int32_t *ee,
                            const uint8_t *ee_isnew, double outer_eta, double inner_eta, double stiffness, double cor,
                            double dt, double *F, uint8_t *vf_fired, uint8_t *ee_fired, int *newused) {
  int rc = check_args(ctx, nverts, q, v, F, n_vf, vf, n_ee, ee);
  if (rc) return rc;
  for (int k = 0; k < 2; k++) {
    const int32_t *st = k == 0 ? vf : ee;
    const int64_t n = k == 0 ? n_vf : n_ee;
    for (int64_t i = 0; i < 4 * n; i++)
      if (st[i] < 0 || st[i] >= nverts) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "stencil vertex out of range");
  }
  if (newused) *newused = 0;
  if (nverts == 0) return CCD_OK;
  CCD_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t s = ctx->stream;
  const int64_t n = n_vf + n_ee, V3 = 3 * (int64_t)nverts;
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    const size_t at = off;
    off += (bytes + 255) / 256 * 256;
    return at;
  };
  const size_t o_q = carve(V3 * 8), o_v = carve(V3 * 8), o_F = carve(V3 * 8);
  const size_t o_st = carve((size_t)16 * std::max<int64_t>(n, 1)), o_new = carve((size_t)std::max<int64_t>(n, 1));
  const size_t o_fired = carve((size_t)std::max<int64_t>(n, 1));
  char *mem = nullptr;
  CCD_CUDA(cudaMallocAsync((void **)&mem, off, s));
  double *d_q = (double *)(mem + o_q), *d_v = (double *)(mem + o_v), *d_F = (double *)(mem + o_F);
  int32_t *d_st = (int32_t *)(mem + o_st);
  uint8_t *d_new = (uint8_t *)(mem + o_new), *d_fired = (uint8_t *)(mem + o_fired);
  auto run = [&]() -> int {
    CCD_CUDA(cudaMemcpyAsync(d_q, q, V3 * 8, cudaMemcpyHostToDevice, s));
    CCD_CUDA(cudaMemcpyAsync(d_v, v, V3 * 8, cudaMemcpyHostToDevice, s));
    CCD_CUDA(cudaMemcpyAsync(d_F, F, V3 * 8, cudaMemcpyHostToDevice, s));
    CCD_CUDA(cudaMemsetAsync(d_new, 0, (size_t)std::max<int64_t>(n, 1), s));
    if (n_vf) CCD_CUDA(cudaMemcpyAsync(d_st, vf, (size_t)n_vf * 16, cudaMemcpyHostToDevice, s));
    if (n_ee) CCD_CUDA(cudaMemcpyAsync(d_st + 4 * n_vf, ee, (size_t)n_ee * 16, cudaMemcpyHostToDevice, s));
    if (n_vf && vf_isnew) CCD_CUDA(cudaMemcpyAsync(d_new, vf_isnew, (size_t)n_vf, cudaMemcpyHostToDevice, s));
    if (n_ee && ee_isnew) CCD_CUDA(cudaMemcpyAsync(d_new + n_vf, ee_isnew, (size_t)n_ee, cudaMemcpyHostToDevice, s));
    const ccd::PenaltyParams pp{outer_eta, inner_eta, stiffness, cor};
    const int r = penalty_device(ctx, nverts, d_q, d_v, n_vf, n_ee, d_st, d_new, pp, dt, d_F, d_fired, newused);
    if (r) return r;
    CCD_CUDA(cudaMemcpyAsync(F, d_F, V3 * 8, cudaMemcpyDeviceToHost, s));
    if (vf_fired && n_vf) CCD_CUDA(cudaMemcpyAsync(vf_fired, d_fired, (size_t)n_vf, cudaMemcpyDeviceToHost, s));
    if (ee_fired && n_ee)
      CCD_CUDA(cudaMemcpyAsync(ee_fired, d_fired + n_vf, (size_t)n_ee, cudaMemcpyDeviceToHost, s));
    CCD_CUDA(cudaStreamSynchronize(s));
    return CCD_OK;
  };
  rc = run();
  cudaFreeAsync(mem, s);
  return rc;
}

}  // extern "C"
