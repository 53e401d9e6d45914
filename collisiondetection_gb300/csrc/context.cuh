// Internal state behind the C ABI, shared by the primitive-batch and mesh
// translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/ccd_gb300.h"
#include "narrow.cuh"
#include "stages.cuh"

namespace ccd_capi {

// Largest chunk of the host-memory batch pipeline (two chunks in flight); a
// batch is cut into equal chunks no larger than this.  Large chunks keep the
// refinement's survivors above the wavefront solver's threshold (smaller
// ones fall back to the slower per-warp solver) and pay its latency-bound
// tail once per chunk: on the 20M-row raw batch, 8M-row chunks run 1.54x
// faster end to end than 1M-row ones.  ccd_context_set_option "chunk_rows"
// changes it per context.
constexpr int64_t kChunkRows = 1 << 23;
// Survivor rows per tile of the staged refinement.  Each tile ends in a
// latency-bound tail (the slowest root solves), so tiles are large: the
// scratch is about 5 KB per survivor row (about 20 GB at this size; a batch
// of n < 2^22 rows allocates for n).
constexpr int64_t kStageTileRows = 1 << 22;

// Scratch of the staged refinement, grown on demand.
struct StageBuf {
  void *mem = nullptr;
  int64_t cap = 0;
  ccd::StageScratch view{};
};

struct Slot {
  double *rows = nullptr;
  double *eta = nullptr;
  uint8_t *hit = nullptr;
  double *t = nullptr;
  int32_t *surv = nullptr;
  ccd::BatchCounters *counters = nullptr;    // device
  ccd::BatchCounters *h_counters = nullptr;  // pinned host
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  int64_t cap = 0;
  StageBuf stage;
};

// Events bracketing the kernels of one batch (profiling only).
struct PhaseEvents {
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  bool used = false;
  bool culled = false;
  int stage_launches = 0;
};

}  // namespace ccd_capi

using ccd_capi::PhaseEvents;
using ccd_capi::Slot;
using ccd_capi::StageBuf;

struct ccd_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  Slot slot[2];
  // scratch for the device-memory entry points
  StageBuf stage;
  int32_t *d_surv = nullptr;
  int64_t surv_cap = 0;
  ccd::BatchCounters *d_counters = nullptr;
  ccd::BatchCounters *h_counters = nullptr;
  // scratch of the distance entry points
  void *dist_mem = nullptr;
  size_t dist_cap = 0;
  bool pending_stats = false;
  ccd_batch_stats last{};
  // per-kernel timing
  bool profiling = false;
  PhaseEvents phase[2];      // host-pipeline slots
  PhaseEvents dev_ring[32];  // device entry points, collected lazily
  int dev_next = 0;
  ccd_batch_timings timings{};
  // tuning options (ccd_context_set_option)
  int opt_wave_steps = ccd::kWaveSteps;
  int64_t opt_wave_min_rows = ccd::kWaveMinRows;
  int opt_pool_budget = ccd::kPoolBudget;
  int opt_warp_finish = 1;  // the slowest root solves run on whole warps
  int opt_pool_slots = 64;     // pool kernel (batches the wavefront does not take): slots per warp, 32 or 64
  int opt_pool_slots_min = 4;  // pool kernel: slots per warp at least (a small batch's jobs spread over warps)
  int opt_pool_all = 0;
  int opt_pool_phase_sync = 16;  // pool kernel: prefer the phase of the SM clock's 2^k-cycle window (0: off)        // pool kernel: solves left that step together once its queue is drained
  int opt_shift_after = 2;  // warp_finish 2: failed shifts of a stage before the rest run at once
  int opt_count_tests = 0;
  int opt_traversal = 3;  // broad-phase traversal (ccd_context_set_option "traversal")
  int opt_tree_refit = 1;         // keep a mesh's tree and refit it while its quality holds
  int opt_tree_rebuild_pct = 130;  // rebuild once the node surface exceeds this percentage of its built value
  int opt_tree_max_refits = 64;    // ... or after this many refits in a row
  int64_t opt_layer_grid_min = 1024;  // velocity filter: groups this large fire over the whole GPU
  int64_t opt_chunk_rows = ccd_capi::kChunkRows;  // host-memory batches: rows per chunk
  // Mesh narrow phase: stencils per chunk.  Each chunk's refinement ends in
  // the latency-bound tail of its slowest root solves, so chunks are large
  // (about 1.3 KB of rows and results per stencil: 22 GB per kind for a step
  // of 2^24 stencils or more, allocated for min(stencils, chunk)).  On the
  // 512-instance batch (167 M stencils) 2^24 takes 12.3 s against 13.7 s
  // at 2^22.
  int64_t opt_narrow_chunk = (int64_t)1 << 24;
  int64_t opt_layer_events = (int64_t)1 << 20;      // velocity filter: firings per event-loop launch
  std::string err;
};


namespace ccd_capi {

inline bool valid_path(int path) {
  return path == CCD_PATH_FP64 || path == CCD_PATH_CULL_REFINE || path == CCD_PATH_REFINE_ALL;
}
int fail(ccd_context *ctx, int code, const std::string &msg);
int cuda_fail(ccd_context *ctx, cudaError_t e, const char *what);
// Grows a staged-refinement scratch to cover min(rows, tile) survivor rows.
int ensure_stage(ccd_context *ctx, StageBuf &sb, int64_t rows, cudaStream_t s);
// Enqueues the kernels of one batch whose buffers are all on the device.
int enqueue_batch(ccd_context *ctx, const ccd::PrimBatch &b, int path, int32_t *surv, StageBuf &stage,
                  cudaStream_t s, PhaseEvents *pe);

}  // namespace ccd_capi

#define CCD_CUDA(call)                                       \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return ccd_capi::cuda_fail(ctx, e_, #call); \
  } while (0)
