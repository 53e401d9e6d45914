// Kernel templates for the primitive narrow phase, one thread per swept
// primitive ("row").  Each narrow_<kind>.cu instantiates them for one kind so
// that the units compile in parallel.
//
// Compiled with --fmad=false: the FP64 path reproduces the reference's
// one-rounding-per-operation arithmetic (see ccd_ctcd64.h).
#pragma once

#include "ccd_ctcd64.h"
#include "ccd_cull32.h"
#include "narrow.cuh"

namespace ccd {
namespace kernels {


constexpr int kThreads = 128;

template <int KIND>
struct RowWidth {
  static constexpr int value = KIND <= 1 ? 24 : (KIND == 2 ? 18 : 12);
};

// Evaluates one row with the FP64 reference-exact tests.
template <int KIND>
__device__ __forceinline__ bool eval_row(const double *__restrict__ rows, int64_t i, double eta, double &t,
                                         uint8_t &st) {
  constexpr int W = RowWidth<KIND>::value;
  double x[W];
  const double *src = rows + i * W;
#pragma unroll
  for (int j = 0; j < W; j++) x[j] = __ldg(src + j);
  if constexpr (KIND == kVF)
    return vf_ctcd(x, eta, t, st);
  else if constexpr (KIND == kEE)
    return ee_ctcd(x, eta, t, st);
  else if constexpr (KIND == kVE)
    return ve_ctcd(x, eta, t, st);
  else
    return vv_ctcd(x, eta, t);
}

__device__ __forceinline__ void flush_counters(BatchCounters *c, unsigned hits, unsigned flags, unsigned surv) {
  unsigned h = __reduce_add_sync(0xffffffffu, hits);
  unsigned f = __reduce_add_sync(0xffffffffu, flags);
  unsigned s = __reduce_add_sync(0xffffffffu, surv);
  if ((threadIdx.x & 31) == 0) {
    if (h) atomicAdd(&c->hits, (unsigned long long)h);
    if (f) atomicAdd(&c->status_flags, (unsigned long long)f);
    if (s) atomicAdd(&c->survivors, (unsigned long long)s);
  }
}

template <int KIND>
__global__ void __launch_bounds__(kThreads) prims_fp64_kernel(PrimBatch b) {
  unsigned hits = 0, flags = 0, surv = 0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // Every thread of a warp runs the same number of iterations so that the
  // warp-wide counter reduction below sees all 32 lanes.
  const int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t warp_base = base - (threadIdx.x & 31);
  for (int64_t w = warp_base; w < b.n; w += stride) {
    int64_t i = w + (threadIdx.x & 31);
    if (i < b.n) {
      double eta = b.eta_per_row ? __ldg(b.eta + i) : __ldg(b.eta);
      double t = 0.0;
      uint8_t st = 0;
      bool h = eval_row<KIND>(b.rows, i, eta, t, st);
      b.hit[i] = h;
      if (h) b.t[i] = t;
      if (b.status) b.status[i] = st;
      hits += h;
      flags += (st != 0);
      surv += 1;
    }
  }
  flush_counters(b.counters, hits, flags, surv);
}

// FP64 evaluation of the rows in a survivor list (count in
// counters->survivors, written by the cull pass on the same stream).
template <int KIND>
__global__ void __launch_bounds__(kThreads) prims_fp64_list_kernel(PrimBatch b, const int32_t *__restrict__ list) {
  unsigned hits = 0, flags = 0;
  const int64_t count = (int64_t)b.counters->survivors;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t warp_base = base - (threadIdx.x & 31);
  for (int64_t w = warp_base; w < count; w += stride) {
    const int64_t r = w + (threadIdx.x & 31);
    if (r < count) {
      const int64_t i = list[r];
      double eta = b.eta_per_row ? __ldg(b.eta + i) : __ldg(b.eta);
      double t = 0.0;
      uint8_t st = 0;
      bool h = eval_row<KIND>(b.rows, i, eta, t, st);
      b.hit[i] = h;
      if (h) b.t[i] = t;
      if (b.status) b.status[i] = st;
      hits += h;
      flags += (st != 0);
    }
  }
  flush_counters(b.counters, hits, flags, 0);
}

// FP32 rejection pass.  Rows that cannot hit get hit = 0; the others are
// compacted into `list` with one atomic per warp (ballot + popc prefix).
template <int KIND>
__global__ void __launch_bounds__(kThreads) prims_cull_kernel(PrimBatch b, int32_t *__restrict__ list) {
  const unsigned lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t warp_base = base - lane;
  for (int64_t w = warp_base; w < b.n; w += stride) {
    int64_t i = w + lane;
    bool keep = false;
    if (i < b.n) {
      constexpr int W = RowWidth<KIND>::value;
      double x[W];
      const double *src = b.rows + i * W;
#pragma unroll
      for (int j = 0; j < W; j++) x[j] = __ldg(src + j);
      double eta = b.eta_per_row ? __ldg(b.eta + i) : __ldg(b.eta);
      bool rej;
      if constexpr (KIND == kVF)
        rej = vf_rejects(x, eta);
      else if constexpr (KIND == kEE)
        rej = ee_rejects(x, eta);
      else
        rej = ve_rejects(x, eta);
      if (rej) {
        b.hit[i] = 0;
        if (b.status) b.status[i] = 0;
      } else {
        keep = true;
      }
    }
    unsigned mask = __ballot_sync(0xffffffffu, keep);
    if (mask) {
      unsigned long long slot = 0;
      int leader = __ffs(mask) - 1;
      if ((int)lane == leader) slot = atomicAdd(&b.counters->survivors, (unsigned long long)__popc(mask));
      slot = __shfl_sync(0xffffffffu, slot, leader);
      if (keep) list[slot + __popc(mask & ((1u << lane) - 1u))] = (int32_t)i;
    }
  }
}

inline int grid_for(int64_t n, int num_sms, int blocks_per_sm) {
  int64_t need = (n + kThreads - 1) / kThreads;
  int64_t cap = (int64_t)num_sms * blocks_per_sm;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}


template <int KIND>
cudaError_t fp64(const PrimBatch &b, int num_sms, cudaStream_t s) {
  prims_fp64_kernel<KIND><<<grid_for(b.n, num_sms, 8), kThreads, 0, s>>>(b);
  return cudaGetLastError();
}
template <int KIND>
cudaError_t fp64_list(const PrimBatch &b, const int32_t *list, int num_sms, cudaStream_t s) {
  prims_fp64_list_kernel<KIND><<<grid_for(b.n, num_sms, 8), kThreads, 0, s>>>(b, list);
  return cudaGetLastError();
}
template <int KIND>
cudaError_t cull(const PrimBatch &b, int32_t *list, int num_sms, cudaStream_t s) {
  prims_cull_kernel<KIND><<<grid_for(b.n, num_sms, 16), kThreads, 0, s>>>(b, list);
  return cudaGetLastError();
}

}  // namespace kernels
}  // namespace ccd
