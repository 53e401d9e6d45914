// C ABI (include/ccd_gb300.h): contexts, primitive batches.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>

#include "context.cuh"

#define CCD_VERSION_NUMBER 100  // 0.1.0

namespace ccd_capi {

int fail(ccd_context *ctx, int code, const std::string &msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int cuda_fail(ccd_context *ctx, cudaError_t e, const char *what) {
  int code = (e == cudaErrorMemoryAllocation) ? CCD_ERR_OUT_OF_MEMORY : CCD_ERR_CUDA;
  return fail(ctx, code, std::string(what) + ": " + cudaGetErrorString(e));
}


int ensure_stage(ccd_context *ctx, StageBuf &sb, int64_t rows, cudaStream_t s) {
  int64_t cap = std::min<int64_t>(std::max<int64_t>(rows, 1), kStageTileRows);
  // The wavefront solver's scratch (about 3 KB per row) only for batches
  // large enough to use it.
  const bool wave = ctx->opt_wave_steps > 0 && rows >= ctx->opt_wave_min_rows;
  if (sb.cap >= cap && (sb.view.wd != nullptr || !wave)) return CCD_OK;
  cap = std::max<int64_t>(cap, sb.cap);
  CCD_CUDA(cudaStreamSynchronize(s));
  cudaFree(sb.mem);
  sb = StageBuf{};
  const size_t stage_bytes = ccd::stage_scratch_bytes(cap);
  CCD_CUDA(cudaMalloc(&sb.mem, stage_bytes + (wave ? ccd::wave_scratch_bytes(cap) : 0)));
  sb.cap = cap;
  sb.view = ccd::stage_scratch_view(sb.mem, cap);
  if (wave) ccd::attach_wave(sb.view, (char *)sb.mem + stage_bytes);
  return CCD_OK;
}

int free_slot(ccd_context *ctx, Slot &s) {
  cudaFree(s.rows);
  cudaFree(s.eta);
  cudaFree(s.hit);
  cudaFree(s.t);
  cudaFree(s.surv);
  cudaFree(s.counters);
  cudaFreeHost(s.h_counters);
  cudaFree(s.stage.mem);
  cudaStream_t stream = s.stream;
  cudaEvent_t done = s.done;
  s = Slot{};
  s.stream = stream;
  s.done = done;
  (void)ctx;
  return CCD_OK;
}

int ensure_slot(ccd_context *ctx, Slot &s, int64_t rows) {
  if (s.cap >= rows) return CCD_OK;
  if (s.stream) CCD_CUDA(cudaStreamSynchronize(s.stream));
  free_slot(ctx, s);
  CCD_CUDA(cudaMalloc(&s.rows, (size_t)rows * 24 * sizeof(double)));
  CCD_CUDA(cudaMalloc(&s.eta, (size_t)rows * sizeof(double)));
  CCD_CUDA(cudaMalloc(&s.hit, (size_t)rows));
  CCD_CUDA(cudaMalloc(&s.t, (size_t)rows * sizeof(double)));
  CCD_CUDA(cudaMalloc(&s.surv, (size_t)rows * sizeof(int32_t)));
  CCD_CUDA(cudaMalloc(&s.counters, sizeof(ccd::BatchCounters)));
  CCD_CUDA(cudaMallocHost(&s.h_counters, sizeof(ccd::BatchCounters)));
  memset(s.h_counters, 0, sizeof(ccd::BatchCounters));
  s.cap = rows;
  return CCD_OK;
}

int check_batch_args(ccd_context *ctx, int kind, int path, int64_t n, const void *rows, const void *eta,
                     int64_t eta_count, const void *hit, const void *t) {
  if (!ctx) return CCD_ERR_INVALID_ARGUMENT;
  if (kind < CCD_VERTEX_FACE || kind > CCD_VERTEX_VERTEX) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "unknown kind");
  if (!valid_path(path)) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "unknown path");
  if (n < 0 || n > INT32_MAX) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "n must be in [0, 2^31)");
  if (n == 0) return CCD_OK;
  if (!rows || !eta || !hit || !t) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null buffer");
  if (eta_count != 1 && eta_count != n) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "eta_count must be 1 or n");
  return CCD_OK;
}

int ensure_phase_events(ccd_context *ctx, PhaseEvents &pe) {
  for (auto &e : pe.ev)
    if (!e) CCD_CUDA(cudaEventCreate(&e));
  return CCD_OK;
}

// Adds the kernel times recorded in pe to ctx->timings (events must be complete).
int collect_phase(ccd_context *ctx, PhaseEvents &pe) {
  if (!pe.used) return CCD_OK;
  float a = 0.f, b = 0.f;
  CCD_CUDA(cudaEventElapsedTime(&a, pe.ev[0], pe.ev[1]));
  if (pe.culled) {
    CCD_CUDA(cudaEventElapsedTime(&b, pe.ev[1], pe.ev[2]));
    ctx->timings.cull_ms += a;
    ctx->timings.refine_ms += b;
    ctx->timings.launches += 1 + pe.stage_launches;
  } else {
    ctx->timings.refine_ms += a;
    ctx->timings.launches += 1;
  }
  pe.used = false;
  return CCD_OK;
}

// Enqueues the kernels of one batch whose buffers are all on the device.
int enqueue_batch(ccd_context *ctx, const ccd::PrimBatch &b, int path, int32_t *surv, StageBuf &stage,
                  cudaStream_t s, PhaseEvents *pe) {
  CCD_CUDA(cudaMemsetAsync(b.counters, 0, sizeof(ccd::BatchCounters), s));
  if (pe) {
    int rc = ensure_phase_events(ctx, *pe);
    if (rc) return rc;
    CCD_CUDA(cudaEventRecord(pe->ev[0], s));
  }
  // The FP32 stage covers vertex-face, edge-edge and vertex-edge rows;
  // vertex-vertex rows (one quadratic) always take the FP64 kernel.
  // CCD_PATH_REFINE_ALL runs the staged refinement of vertex-face and
  // edge-edge rows on a list of every row instead of the cull's survivors.
  const bool all = path == CCD_PATH_REFINE_ALL && (b.kind == CCD_VERTEX_FACE || b.kind == CCD_EDGE_EDGE);
  bool culled = !(path == CCD_PATH_FP64 || b.kind == CCD_VERTEX_VERTEX) && (path != CCD_PATH_REFINE_ALL || all);
  if (!culled) {
    CCD_CUDA(ccd::launch_prims_fp64(b, ctx->num_sms, s));
    if (pe) CCD_CUDA(cudaEventRecord(pe->ev[1], s));
  } else if (all) {
    int rc = ensure_stage(ctx, stage, b.n, s);
    if (rc) return rc;
    CCD_CUDA(ccd::launch_all_rows(b, surv, s));
    if (pe) CCD_CUDA(cudaEventRecord(pe->ev[1], s));
    int launches = 0;
    ccd::StageScratch view = stage.view;
    view.wave_steps = view.wd ? ctx->opt_wave_steps : 0;
    view.wave_min_rows = ctx->opt_wave_min_rows;
    view.pool_budget = ctx->opt_pool_budget;
    view.warp_finish = ctx->opt_warp_finish;
    view.shift_after = ctx->opt_shift_after;
    view.pool_slots = ctx->opt_pool_slots;
    view.pool_slots_min = ctx->opt_pool_slots_min;
    view.pool_all = ctx->opt_pool_all;
    view.pool_phase_sync = ctx->opt_pool_phase_sync;
    CCD_CUDA(ccd::launch_stages(b, surv, view, ctx->num_sms, s, &launches));
    if (pe) CCD_CUDA(cudaEventRecord(pe->ev[2], s));
    if (pe) pe->stage_launches = launches;
  } else if (b.kind == CCD_VERTEX_EDGE) {
    CCD_CUDA(ccd::launch_prims_cull(b, surv, ctx->num_sms, s));
    if (pe) CCD_CUDA(cudaEventRecord(pe->ev[1], s));
    CCD_CUDA(ccd::launch_prims_fp64_list(b, surv, ctx->num_sms, s));
    if (pe) CCD_CUDA(cudaEventRecord(pe->ev[2], s));
    if (pe) pe->stage_launches = 1;
  } else {
    int rc = ensure_stage(ctx, stage, b.n, s);
    if (rc) return rc;
    CCD_CUDA(ccd::launch_prims_cull(b, surv, ctx->num_sms, s));
    if (pe) CCD_CUDA(cudaEventRecord(pe->ev[1], s));
    int launches = 0;
    ccd::StageScratch view = stage.view;
    view.wave_steps = view.wd ? ctx->opt_wave_steps : 0;
    view.wave_min_rows = ctx->opt_wave_min_rows;
    view.pool_budget = ctx->opt_pool_budget;
    view.warp_finish = ctx->opt_warp_finish;
    view.shift_after = ctx->opt_shift_after;
    view.pool_slots = ctx->opt_pool_slots;
    view.pool_slots_min = ctx->opt_pool_slots_min;
    view.pool_all = ctx->opt_pool_all;
    view.pool_phase_sync = ctx->opt_pool_phase_sync;
    CCD_CUDA(ccd::launch_stages(b, surv, view, ctx->num_sms, s, &launches));
    if (pe) CCD_CUDA(cudaEventRecord(pe->ev[2], s));
    if (pe) pe->stage_launches = launches;
  }
  if (pe) {
    pe->used = true;
    pe->culled = culled;
  }
  return CCD_OK;
}

void add_stats(ccd_batch_stats &st, const ccd::BatchCounters &c) {
  st.survivors += (int64_t)c.survivors;
  st.hits += (int64_t)c.hits;
  st.status_flags += (int64_t)c.status_flags;
}

}  // namespace ccd_capi

using namespace ccd_capi;

extern "C" {

int ccd_version(void) { return CCD_VERSION_NUMBER; }

const char *ccd_status_string(int status) {
  switch (status) {
    case CCD_OK: return "ok";
    case CCD_ERR_INVALID_ARGUMENT: return "invalid argument";
    case CCD_ERR_CUDA: return "CUDA error";
    case CCD_ERR_OUT_OF_MEMORY: return "out of device memory";
    case CCD_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

int ccd_context_create(int device, ccd_context **out) {
  if (!out) return CCD_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return CCD_ERR_NO_DEVICE;
  if (device < 0 || device >= count) return CCD_ERR_INVALID_ARGUMENT;
  ccd_context *ctx = new (std::nothrow) ccd_context();
  if (!ctx) return CCD_ERR_OUT_OF_MEMORY;
  ctx->device = device;
  int rc = CCD_OK;
  do {
    cudaError_t e;
    if ((e = cudaSetDevice(device)) != cudaSuccess) { rc = cuda_fail(ctx, e, "cudaSetDevice"); break; }
    if ((e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) {
      rc = cuda_fail(ctx, e, "cudaDeviceGetAttribute");
      break;
    }
    if ((e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking)) != cudaSuccess) {
      rc = cuda_fail(ctx, e, "cudaStreamCreate");
      break;
    }
    ctx->stream = ctx->own_stream;
    for (auto &s : ctx->slot) {
      if ((e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking)) != cudaSuccess ||
          (e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming)) != cudaSuccess) {
        rc = cuda_fail(ctx, e, "stream/event create");
        break;
      }
    }
    if (rc) break;
    if ((e = cudaMalloc(&ctx->d_counters, sizeof(ccd::BatchCounters))) != cudaSuccess ||
        (e = cudaMallocHost(&ctx->h_counters, sizeof(ccd::BatchCounters))) != cudaSuccess) {
      rc = cuda_fail(ctx, e, "counter alloc");
      break;
    }
    memset(ctx->h_counters, 0, sizeof(ccd::BatchCounters));
  } while (0);
  if (rc) {
    ccd_context_destroy(ctx);
    return rc;
  }
  *out = ctx;
  return CCD_OK;
}

int ccd_context_destroy(ccd_context *ctx) {
  if (!ctx) return CCD_OK;
  cudaSetDevice(ctx->device);
  for (auto &s : ctx->slot) {
    if (s.stream) cudaStreamSynchronize(s.stream);
    free_slot(ctx, s);
    if (s.done) cudaEventDestroy(s.done);
    if (s.stream) cudaStreamDestroy(s.stream);
  }
  if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
  if (ctx->stream && ctx->stream != ctx->own_stream) cudaStreamSynchronize(ctx->stream);
  for (auto &pe : ctx->phase)
    for (auto &e : pe.ev)
      if (e) cudaEventDestroy(e);
  for (auto &pe : ctx->dev_ring)
    for (auto &e : pe.ev)
      if (e) cudaEventDestroy(e);
  cudaFree(ctx->stage.mem);
  cudaFree(ctx->d_surv);
  cudaFree(ctx->d_counters);
  cudaFree(ctx->dist_mem);
  cudaFreeHost(ctx->h_counters);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return CCD_OK;
}

int ccd_context_set_stream(ccd_context *ctx, void *stream) {
  if (!ctx) return CCD_ERR_INVALID_ARGUMENT;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return CCD_OK;
}

int ccd_context_synchronize(ccd_context *ctx) {
  if (!ctx) return CCD_ERR_INVALID_ARGUMENT;
  CCD_CUDA(cudaSetDevice(ctx->device));
  CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (ctx->pending_stats) {
    ctx->last.survivors = (int64_t)ctx->h_counters->survivors;
    ctx->last.hits = (int64_t)ctx->h_counters->hits;
    ctx->last.status_flags = (int64_t)ctx->h_counters->status_flags;
    ctx->pending_stats = false;
  }
  for (auto &pe : ctx->dev_ring) {
    int rc = collect_phase(ctx, pe);
    if (rc) return rc;
  }
  return CCD_OK;
}

int ccd_context_set_profiling(ccd_context *ctx, int on) {
  if (!ctx) return CCD_ERR_INVALID_ARGUMENT;
  int rc = ccd_context_synchronize(ctx);
  if (rc) return rc;
  ctx->profiling = on != 0;
  ctx->timings = ccd_batch_timings{};
  return CCD_OK;
}

int ccd_context_set_option(ccd_context *ctx, const char *name, int64_t value) {
  if (!ctx) return CCD_ERR_INVALID_ARGUMENT;
  if (!name) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null option name");
  const std::string key(name);
  if (key == "wave_steps") {
    if (value < 0 || value > 4096) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "wave_steps must be in [0, 4096]");
    ctx->opt_wave_steps = (int)value;
  } else if (key == "pool_budget") {
    if (value < 0 || value > (1 << 20)) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "pool_budget must be in [0, 2^20]");
    ctx->opt_pool_budget = (int)value;
  } else if (key == "count_slab_tests") {
    if (value < 0 || value > 1) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "count_slab_tests must be 0 or 1");
    ctx->opt_count_tests = (int)value;
  } else if (key == "pool_slots") {
    if (value != 32 && value != 64) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "pool_slots must be 32 or 64");
    ctx->opt_pool_slots = (int)value;
  } else if (key == "pool_slots_min") {
    if (value < 1 || value > 64) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "pool_slots_min must be in [1, 64]");
    ctx->opt_pool_slots_min = (int)value;
  } else if (key == "pool_phase_sync") {
    if (value < 0 || value > 30) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "pool_phase_sync must be in [0, 30]");
    ctx->opt_pool_phase_sync = (int)value;
  } else if (key == "pool_all") {
    if (value < 0 || value > 32) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "pool_all must be in [0, 32]");
    ctx->opt_pool_all = (int)value;
  } else if (key == "shift_after") {
    if (value < 0 || value > 19) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "shift_after must be in [0, 19]");
    ctx->opt_shift_after = (int)value;
  } else if (key == "warp_finish") {
    if (value < 0 || value > 2) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "warp_finish must be 0, 1 or 2");
    ctx->opt_warp_finish = (int)value;
  } else if (key == "tree_refit") {
    if (value < 0 || value > 1) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "tree_refit must be 0 or 1");
    ctx->opt_tree_refit = (int)value;
  } else if (key == "tree_rebuild_pct") {
    if (value < 100 || value > 100000) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "tree_rebuild_pct must be in [100, 100000]");
    ctx->opt_tree_rebuild_pct = (int)value;
  } else if (key == "tree_max_refits") {
    if (value < 0 || value > (1 << 20)) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "tree_max_refits must be in [0, 2^20]");
    ctx->opt_tree_max_refits = (int)value;
  } else if (key == "traversal") {
    if (value < 0 || value > 4) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "traversal must be in [0, 4]");
    ctx->opt_traversal = (int)value;
  } else if (key == "wave_min_rows") {
    if (value < 0) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "wave_min_rows must be >= 0");
    ctx->opt_wave_min_rows = value;
  } else if (key == "chunk_rows") {
    if (value < 1024 || value > ((int64_t)1 << 26))
      return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "chunk_rows must be in [1024, 2^26]");
    ctx->opt_chunk_rows = value;
  } else if (key == "narrow_chunk") {
    if (value < 1024 || value > ((int64_t)1 << 24))
      return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "narrow_chunk must be in [1024, 2^24]");
    ctx->opt_narrow_chunk = value;
  } else if (key == "layer_events_per_launch") {
    if (value < 1) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "layer_events_per_launch must be >= 1");
    ctx->opt_layer_events = value;
  } else if (key == "layer_grid_min") {
    if (value < 1) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "layer_grid_min must be >= 1");
    ctx->opt_layer_grid_min = value;
  } else {
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "unknown option " + key);
  }
  return CCD_OK;
}

int ccd_last_batch_timings(ccd_context *ctx, ccd_batch_timings *out) {
  if (!ctx || !out) return CCD_ERR_INVALID_ARGUMENT;
  *out = ctx->timings;
  return CCD_OK;
}

const char *ccd_last_error(const ccd_context *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int ccd_last_batch_stats(const ccd_context *ctx, ccd_batch_stats *out) {
  if (!ctx || !out) return CCD_ERR_INVALID_ARGUMENT;
  *out = ctx->last;
  return CCD_OK;
}

int ccd_prim_batch_device(ccd_context *ctx, int kind, int path, int64_t n, const double *rows, const double *eta,
                          int64_t eta_count, uint8_t *hit, double *t, uint8_t *status) {
  int rc = check_batch_args(ctx, kind, path, n, rows, eta, eta_count, hit, t);
  if (rc) return rc;
  ctx->last = ccd_batch_stats{};
  ctx->last.rows = n;
  if (n == 0) return CCD_OK;
  CCD_CUDA(cudaSetDevice(ctx->device));
  if (path != CCD_PATH_FP64 && ctx->surv_cap < n) {
    CCD_CUDA(cudaStreamSynchronize(ctx->stream));
    cudaFree(ctx->d_surv);
    ctx->d_surv = nullptr;
    ctx->surv_cap = 0;
    CCD_CUDA(cudaMalloc(&ctx->d_surv, (size_t)n * sizeof(int32_t)));
    ctx->surv_cap = n;
  }
  PhaseEvents *pe = nullptr;
  if (ctx->profiling) {
    pe = &ctx->dev_ring[ctx->dev_next];
    ctx->dev_next = (ctx->dev_next + 1) % 32;
    if (pe->used) {  // a batch 32 calls back still holds this slot
      CCD_CUDA(cudaEventSynchronize(pe->ev[pe->culled ? 2 : 1]));
      rc = collect_phase(ctx, *pe);
      if (rc) return rc;
    }
  }
  ccd::PrimBatch b{kind, n, rows, eta, eta_count == n && n != 1, hit, t, status, ctx->d_counters};
  rc = enqueue_batch(ctx, b, path, ctx->d_surv, ctx->stage, ctx->stream, pe);
  if (rc) return rc;
  CCD_CUDA(cudaMemcpyAsync(ctx->h_counters, ctx->d_counters, sizeof(ccd::BatchCounters), cudaMemcpyDeviceToHost,
                           ctx->stream));
  ctx->pending_stats = true;
  return CCD_OK;
}

int ccd_prim_cull_device(ccd_context *ctx, int kind, int64_t n, const double *rows, const double *eta,
                         int64_t eta_count, uint8_t *hit, int32_t *survivors, int64_t *n_survivors) {
  if (!ctx) return CCD_ERR_INVALID_ARGUMENT;
  if (!n_survivors) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null survivor count");
  *n_survivors = 0;
  if (kind != CCD_VERTEX_FACE && kind != CCD_EDGE_EDGE && kind != CCD_VERTEX_EDGE)
    return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "the FP32 stage takes vertex-face, edge-edge and vertex-edge rows");
  if (n < 0 || n > INT32_MAX) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "n must be in [0, 2^31)");
  if (n == 0) return CCD_OK;
  if (!rows || !eta || !hit || !survivors) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null buffer");
  if (eta_count != 1 && eta_count != n) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "eta_count must be 1 or n");
  CCD_CUDA(cudaSetDevice(ctx->device));
  ccd::PrimBatch b{kind, n, rows, eta, eta_count == n && n != 1, hit, nullptr, nullptr, ctx->d_counters};
  CCD_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(ccd::BatchCounters), ctx->stream));
  CCD_CUDA(ccd::launch_prims_cull(b, survivors, ctx->num_sms, ctx->stream));
  CCD_CUDA(cudaMemcpyAsync(ctx->h_counters, ctx->d_counters, sizeof(ccd::BatchCounters), cudaMemcpyDeviceToHost,
                           ctx->stream));
  CCD_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->pending_stats = false;
  ctx->last = ccd_batch_stats{};
  ctx->last.rows = n;
  ctx->last.survivors = (int64_t)ctx->h_counters->survivors;
  *n_survivors = ctx->last.survivors;
  return CCD_OK;
}

int ccd_prim_batch(ccd_context *ctx, int kind, int path, int64_t n, const double *rows, const double *eta,
                   int64_t eta_count, uint8_t *hit, double *t) {
  int rc = check_batch_args(ctx, kind, path, n, rows, eta, eta_count, hit, t);
  if (rc) return rc;
  ctx->last = ccd_batch_stats{};
  ctx->last.rows = n;
  if (n == 0) return CCD_OK;
  CCD_CUDA(cudaSetDevice(ctx->device));
  const int W = ccd::row_width(kind);
  const int64_t pieces = (n + ctx->opt_chunk_rows - 1) / ctx->opt_chunk_rows;
  const int64_t chunk = (n + pieces - 1) / pieces;  // equal chunks, none small
  for (auto &s : ctx->slot) {
    rc = ensure_slot(ctx, s, chunk);
    if (rc) return rc;
  }
  const bool per_row = (eta_count == n && n != 1);
  ctx->phase[0].used = ctx->phase[1].used = false;
  int64_t nchunks = (n + chunk - 1) / chunk;
  for (int64_t c = 0; c < nchunks; c++) {
    Slot &s = ctx->slot[c & 1];
    const int64_t off = c * chunk;
    const int64_t m = std::min<int64_t>(chunk, n - off);
    if (c >= 2) {
      // The slot's previous chunk must be fully copied out before reuse.
      CCD_CUDA(cudaEventSynchronize(s.done));
      add_stats(ctx->last, *s.h_counters);
      rc = collect_phase(ctx, ctx->phase[c & 1]);
      if (rc) return rc;
    }
    CCD_CUDA(cudaMemcpyAsync(s.rows, rows + off * W, (size_t)m * W * sizeof(double), cudaMemcpyHostToDevice,
                             s.stream));
    CCD_CUDA(cudaMemcpyAsync(s.eta, per_row ? eta + off : eta, (size_t)(per_row ? m : 1) * sizeof(double),
                             cudaMemcpyHostToDevice, s.stream));
    // t is written only where hit: start from the caller's values.
    CCD_CUDA(cudaMemcpyAsync(s.t, t + off, (size_t)m * sizeof(double), cudaMemcpyHostToDevice, s.stream));
    ccd::PrimBatch b{kind, m, s.rows, s.eta, per_row, s.hit, s.t, nullptr, s.counters};
    rc = enqueue_batch(ctx, b, path, s.surv, s.stage, s.stream, ctx->profiling ? &ctx->phase[c & 1] : nullptr);
    if (rc) return rc;
    CCD_CUDA(cudaMemcpyAsync(hit + off, s.hit, (size_t)m, cudaMemcpyDeviceToHost, s.stream));
    CCD_CUDA(cudaMemcpyAsync(t + off, s.t, (size_t)m * sizeof(double), cudaMemcpyDeviceToHost, s.stream));
    CCD_CUDA(cudaMemcpyAsync(s.h_counters, s.counters, sizeof(ccd::BatchCounters), cudaMemcpyDeviceToHost,
                             s.stream));
    CCD_CUDA(cudaEventRecord(s.done, s.stream));
  }
  for (int64_t c = std::max<int64_t>(0, nchunks - 2); c < nchunks; c++) {
    Slot &s = ctx->slot[c & 1];
    CCD_CUDA(cudaEventSynchronize(s.done));
    add_stats(ctx->last, *s.h_counters);
    rc = collect_phase(ctx, ctx->phase[c & 1]);
    if (rc) return rc;
  }
  return CCD_OK;
}

static int single(ccd_context *ctx, int kind, const double *points, double eta, int *hit, double *t) {
  if (!ctx || !points || !hit || !t) return fail(ctx, CCD_ERR_INVALID_ARGUMENT, "null argument");
  uint8_t h = 0;
  double tt = *t;
  int rc = ccd_prim_batch(ctx, kind, CCD_PATH_FP64, 1, points, &eta, 1, &h, &tt);
  if (rc) return rc;
  *hit = h;
  if (h) *t = tt;
  return CCD_OK;
}

int ccd_vertex_face_ctcd(ccd_context *ctx, const double *p, double eta, int *hit, double *t) {
  return single(ctx, CCD_VERTEX_FACE, p, eta, hit, t);
}
int ccd_edge_edge_ctcd(ccd_context *ctx, const double *p, double eta, int *hit, double *t) {
  return single(ctx, CCD_EDGE_EDGE, p, eta, hit, t);
}
int ccd_vertex_edge_ctcd(ccd_context *ctx, const double *p, double eta, int *hit, double *t) {
  return single(ctx, CCD_VERTEX_EDGE, p, eta, hit, t);
}
int ccd_vertex_vertex_ctcd(ccd_context *ctx, const double *p, double eta, int *hit, double *t) {
  return single(ctx, CCD_VERTEX_VERTEX, p, eta, hit, t);
}

}  // extern "C"
