// Work-split autotuner of the staged refinement (C ABI: ccd_autotune_prim_batch).
//
// The refinement of a large vertex-face or edge-edge batch splits its root
// solves between a lock-step wavefront (wave_steps launches over every queued
// polynomial), a pool kernel that packs the unfinished solves many per warp
// (pool_budget steps each), and a one-per-warp finish of the last ones (on
// all lanes of the warp, or with a stage's remaining shifts tried at once,
// warp_finish / shift_after); batches below wave_min_rows skip the wavefront.  Which split is fastest depends on
// the batch (how many rows survive the cull, how many solves run long) and on
// the GPU, so the tuner times each candidate split on the caller's own rows
// and keeps the fastest.  A split changes only the schedule of the solves,
// never their arithmetic: every candidate's hits and contact times are
// compared bit for bit with the first run's, and a candidate that differs is
// counted and never chosen.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "context.cuh"

namespace {

// Counts the rows whose hit flag differs, or whose contact time differs bit
// for bit where both hit.
__global__ void count_mismatches(const uint8_t *h0, const double *t0, const uint8_t *h1, const double *t1,
                                 int64_t n, unsigned long long *out) {
  unsigned bad = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const bool h = h0[i] != 0;
    bad += (h != (h1[i] != 0)) ||
           (h && __double_as_longlong(t0[i]) != __double_as_longlong(t1[i]));
  }
  bad = __reduce_add_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0 && bad) atomicAdd(out, (unsigned long long)bad);
}

struct Split {
  int wave_steps;
  int pool_budget;
  int warp_finish;
  int shift_after;
};

struct TuneBuffers {
  uint8_t *hit[2] = {nullptr, nullptr};
  double *t[2] = {nullptr, nullptr};
  unsigned long long *bad = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~TuneBuffers() {
    for (int k = 0; k < 2; k++) {
      cudaFree(hit[k]);
      cudaFree(t[k]);
      if (ev[k]) cudaEventDestroy(ev[k]);
    }
    cudaFree(bad);
  }
};

// FP64 throughput probe: every thread runs kChains independent chains of
// x = x * a + b, as a DMUL and a DADD (the library is built without FMA
// contraction) or as one DFMA.  a is just below 1 and b small, so the chains
// stay finite and normal.  The sum is stored only if it equals an impossible
// value, which keeps the chains live without a store per thread.
constexpr int kPeakThreads = 256;
constexpr int kChains = 8;

template <bool FMA>
__global__ void __launch_bounds__(kPeakThreads) fp64_chains(int iters, double a, double b, double *sink) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) x[k] = 1.0 + 1e-3 * (double)(threadIdx.x + k);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < kChains; k++) {
      if (FMA) {
        x[k] = __fma_rn(x[k], a, b);
      } else {
        x[k] = x[k] * a;
        x[k] = x[k] + b;
      }
    }
  }
  double sum = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; k++) sum += x[k];
  if (sum == -1.0) sink[0] = sum;
}

// Division throughput: kChains independent chains x = c / x per thread
// (c near 1.3, so every x stays near 1).
__global__ void __launch_bounds__(kPeakThreads) fp64_div_chains(int iters, double c, double *sink) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) x[k] = 1.0 + 1e-3 * (double)(threadIdx.x + k);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = c / x[k];
  }
  double sum = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; k++) sum += x[k];
  if (sum == -1.0) sink[0] = sum;
}

// Latency: one warp runs one dependent chain of each operation, timed with
// the SM clock.  cycles[0..2] = add, multiply, division chain lengths in
// cycles; the host divides by the chain length.
__global__ void fp64_latency(int iters, double a, double b, double c, double *sink, long long *cycles) {
  double x = 1.0 + 1e-3 * (double)threadIdx.x;
  __syncwarp();
  const long long t0 = clock64();
  for (int i = 0; i < iters; i++) x = x + b;
  const long long t1 = clock64();
  for (int i = 0; i < iters; i++) x = x * a;
  const long long t2 = clock64();
  for (int i = 0; i < iters; i++) x = c / x;
  const long long t3 = clock64();
  if (x == -1.0) sink[0] = x;
  if (threadIdx.x == 0) {
    cycles[0] = t1 - t0;
    cycles[1] = t2 - t1;
    cycles[2] = t3 - t2;
  }
}

}  // namespace

using namespace ccd_capi;

extern "C" {

int ccd_autotune_prim_batch(ccd_context *ctx, int kind, int64_t n, const double *rows, const double *eta,
                            int64_t eta_count, int reps, ccd_tune_result *out) {
  if (!ctx) return CCD_ERR_INVALID_ARGUMENT;
  if (!out) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null result");
  if (kind != CCD_VERTEX_FACE && kind != CCD_EDGE_EDGE)
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "only vertex-face and edge-edge batches have a staged refinement");
  if (n <= 0 || n > INT32_MAX) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "n must be in [1, 2^31)");
  if (!rows || !eta) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null buffer");
  if (eta_count != 1 && eta_count != n) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "eta_count must be 1 or n");
  if (reps < 1 || reps > 64) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "reps must be in [1, 64]");
  *out = ccd_tune_result{};
  CCD_CUDA(cudaSetDevice(ctx->device));
  CCD_CUDA(cudaStreamSynchronize(ctx->stream));

  TuneBuffers tb;
  for (int k = 0; k < 2; k++) {
    CCD_CUDA(cudaMalloc(&tb.hit[k], (size_t)n));
    CCD_CUDA(cudaMalloc(&tb.t[k], (size_t)n * sizeof(double)));
    CCD_CUDA(cudaEventCreate(&tb.ev[k]));
  }
  CCD_CUDA(cudaMalloc(&tb.bad, sizeof(unsigned long long)));

  // Restores the context's options on every early return; the chosen split
  // is committed at the end.
  struct Saved {
    ccd_context *ctx;
    int steps, budget, finish, after;
    int64_t min_rows;
    bool profiling, committed = false;
    ~Saved() {
      ctx->profiling = profiling;
      if (committed) return;
      ctx->opt_wave_steps = steps;
      ctx->opt_pool_budget = budget;
      ctx->opt_warp_finish = finish;
      ctx->opt_shift_after = after;
      ctx->opt_wave_min_rows = min_rows;
    }
  } saved{ctx,          ctx->opt_wave_steps,     ctx->opt_pool_budget, ctx->opt_warp_finish,
          ctx->opt_shift_after, ctx->opt_wave_min_rows, ctx->profiling};
  const int saved_steps = saved.steps, saved_budget = saved.budget;
  const int saved_finish = saved.finish, saved_after = saved.after;
  const int64_t saved_min_rows = saved.min_rows;
  ctx->profiling = false;

  // The context's own settings come first: their output is the one every
  // other candidate must reproduce.  Then the pool kernel alone, then the
  // wavefront at each step count with each pool budget, then short pool
  // budgets whose leftovers finish one per warp with their stages' remaining
  // shifts tried at once.
  std::vector<Split> cands;
  cands.push_back({n >= saved_min_rows ? saved_steps : 0, saved_budget, saved_finish, saved_after});
  cands.push_back({0, 0, saved_finish, saved_after});
  for (int steps : {16, 32, 48, 64, 96, 128})
    for (int budget : {0, 256, 4096}) cands.push_back({steps, budget, saved_finish, saved_after});
  for (int steps : {32, 48, 64})
    for (int budget : {64, 256}) cands.push_back({steps, budget, 2, 1});

  // One run of the batch under the current options into output set k, with
  // the contact times starting as NaN (t is written only where hit).
  auto run = [&](int k, float *ms) -> int {
    CCD_CUDA(cudaMemsetAsync(tb.t[k], 0xff, (size_t)n * sizeof(double), ctx->stream));
    CCD_CUDA(cudaEventRecord(tb.ev[0], ctx->stream));
    int rc = ccd_prim_batch_device(ctx, kind, CCD_PATH_CULL_REFINE, n, rows, eta, eta_count, tb.hit[k], tb.t[k],
                                   nullptr);
    if (rc) return rc;
    CCD_CUDA(cudaEventRecord(tb.ev[1], ctx->stream));
    CCD_CUDA(cudaEventSynchronize(tb.ev[1]));
    if (ms) CCD_CUDA(cudaEventElapsedTime(ms, tb.ev[0], tb.ev[1]));
    return CCD_OK;
  };

  // Median time of one split (after a warm-up run, which also grows the
  // scratch outside the timing) into output set k; for k = 1, *bad receives
  // the rows that differ from set 0.
  auto time_split = [&](const Split &c, int k, double *med, unsigned long long *bad) -> int {
    // The wavefront runs only for batches of at least wave_min_rows rows.
    ctx->opt_wave_steps = c.wave_steps;
    ctx->opt_pool_budget = c.pool_budget;
    ctx->opt_warp_finish = c.warp_finish;
    ctx->opt_shift_after = c.shift_after;
    ctx->opt_wave_min_rows = std::min<int64_t>(saved_min_rows, n);
    int rc = run(k, nullptr);
    std::vector<float> times;
    for (int r = 0; !rc && r < reps; r++) {
      float ms = 0.f;
      rc = run(k, &ms);
      times.push_back(ms);
    }
    if (rc) return rc;
    std::sort(times.begin(), times.end());
    *med = times[times.size() / 2];
    *bad = 0;
    if (k == 1) {
      CCD_CUDA(cudaMemsetAsync(tb.bad, 0, sizeof(unsigned long long), ctx->stream));
      count_mismatches<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(tb.hit[0], tb.t[0], tb.hit[1], tb.t[1], n,
                                                                  tb.bad);
      CCD_CUDA(cudaGetLastError());
      CCD_CUDA(cudaMemcpyAsync(bad, tb.bad, sizeof(*bad), cudaMemcpyDeviceToHost, ctx->stream));
      CCD_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return CCD_OK;
  };

  double best_ms = 0.0;
  Split best{};
  int best_i = -1;
  for (size_t i = 0; i < cands.size(); i++) {
    double med = 0.0;
    unsigned long long bad = 0;
    int rc = time_split(cands[i], i == 0 ? 0 : 1, &med, &bad);
    if (rc) return rc;
    out->candidates++;
    if (i == 0) out->default_ms = med;
    if (bad) {
      out->mismatches++;
      continue;
    }
    if (best_i < 0 || med < best_ms) {
      best_ms = med;
      best = cands[i];
      best_i = (int)i;
    }
  }
  // The first split is timed first, before the GPU has run this batch for
  // long; on GB300 its edge-edge median came out about 5% slower than the
  // same split timed later in the sweep.  Time it once more at the end and
  // keep its faster median.
  {
    double med = 0.0;
    unsigned long long bad = 0;
    int rc = time_split(cands[0], 1, &med, &bad);
    if (rc) return rc;
    if (bad) {
      out->mismatches++;
    } else {
      out->default_ms = std::min(out->default_ms, med);
      if (best_i != 0 && med <= best_ms) {
        best_ms = med;
        best = cands[0];
        best_i = 0;
      } else if (best_i == 0) {
        best_ms = out->default_ms;
      }
    }
  }

  out->best_ms = best_ms;
  saved.committed = true;
  if (best.wave_steps > 0) {
    // Batches as large as this one take the wavefront with the chosen split.
    ctx->opt_wave_steps = best.wave_steps;
    ctx->opt_pool_budget = best.pool_budget;
    ctx->opt_warp_finish = best.warp_finish;
    ctx->opt_shift_after = best.shift_after;
    ctx->opt_wave_min_rows = std::min<int64_t>(saved_min_rows, n);
  } else {
    // The pool kernel alone won: batches up to this size skip the wavefront;
    // larger ones keep the context's split.
    ctx->opt_wave_steps = saved_steps;
    ctx->opt_pool_budget = saved_budget;
    ctx->opt_warp_finish = saved_finish;
    ctx->opt_shift_after = saved_after;
    ctx->opt_wave_min_rows = std::max<int64_t>(saved_min_rows, n + 1);
  }
  out->wave_steps = ctx->opt_wave_steps;
  out->pool_budget = ctx->opt_pool_budget;
  out->warp_finish = ctx->opt_warp_finish;
  out->shift_after = ctx->opt_shift_after;
  out->wave_min_rows = ctx->opt_wave_min_rows;
  out->chosen = best_i;
  return CCD_OK;
}

int ccd_fp64_peak(ccd_context *ctx, int reps, ccd_fp64_peak_result *out) {
  if (!ctx) return CCD_ERR_INVALID_ARGUMENT;
  if (!out) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null result");
  if (reps < 1 || reps > 64) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "reps must be in [1, 64]");
  *out = ccd_fp64_peak_result{};
  CCD_CUDA(cudaSetDevice(ctx->device));
  int per_sm = 0;
  CCD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fp64_chains<false>, kPeakThreads, 0));
  const int grid = ctx->num_sms * std::max(1, per_sm);
  const int iters = 4096;
  double *sink = nullptr;
  long long *cycles = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  struct Cleanup {
    double *&sink;
    long long *&cycles;
    cudaEvent_t *ev;
    ~Cleanup() {
      cudaFree(sink);
      cudaFree(cycles);
      for (int k = 0; k < 2; k++)
        if (ev[k]) cudaEventDestroy(ev[k]);
    }
  } cleanup{sink, cycles, ev};
  CCD_CUDA(cudaMalloc(&sink, sizeof(double)));
  CCD_CUDA(cudaMalloc(&cycles, 3 * sizeof(long long)));
  for (int k = 0; k < 2; k++) CCD_CUDA(cudaEventCreate(&ev[k]));
  const double a = 0.9999999, b = 1e-7, c = 1.3;
  const int div_iters = iters / 8;
  float best[3] = {0.f, 0.f, 0.f};
  for (int kind = 0; kind < 3; kind++) {  // add + multiply, fused multiply-add, division
    for (int r = 0; r <= reps; r++) {     // the first run warms up
      CCD_CUDA(cudaEventRecord(ev[0], ctx->stream));
      if (kind == 1)
        fp64_chains<true><<<grid, kPeakThreads, 0, ctx->stream>>>(iters, a, b, sink);
      else if (kind == 0)
        fp64_chains<false><<<grid, kPeakThreads, 0, ctx->stream>>>(iters, a, b, sink);
      else
        fp64_div_chains<<<grid, kPeakThreads, 0, ctx->stream>>>(div_iters, c, sink);
      CCD_CUDA(cudaGetLastError());
      CCD_CUDA(cudaEventRecord(ev[1], ctx->stream));
      CCD_CUDA(cudaEventSynchronize(ev[1]));
      float ms = 0.f;
      CCD_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
      if (r > 0 && (best[kind] == 0.f || ms < best[kind])) best[kind] = ms;
    }
  }
  const double lanes = (double)grid * kPeakThreads * kChains * iters;
  out->ops = (int64_t)(2.0 * lanes);
  out->ms = best[0];
  out->ops_per_s = 2.0 * lanes / (best[0] * 1e-3);
  out->fma_flops_per_s = 2.0 * lanes / (best[1] * 1e-3);
  out->div_per_s = (double)grid * kPeakThreads * kChains * div_iters / (best[2] * 1e-3);
  const int lat_iters = 2048;
  for (int r = 0; r < 2; r++) {  // the first run warms up
    fp64_latency<<<1, 32, 0, ctx->stream>>>(lat_iters, a, b, c, sink, cycles);
    CCD_CUDA(cudaGetLastError());
  }
  long long host_cycles[3] = {0, 0, 0};
  CCD_CUDA(cudaMemcpyAsync(host_cycles, cycles, sizeof host_cycles, cudaMemcpyDeviceToHost, ctx->stream));
  CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  out->add_latency_cycles = (double)host_cycles[0] / lat_iters;
  out->mul_latency_cycles = (double)host_cycles[1] / lat_iters;
  out->div_latency_cycles = (double)host_cycles[2] / lat_iters;
  return CCD_OK;
}

}  // extern "C"
