// Staged FP64 refinement (stages.cuh): scratch layout and the launchers for
// vertex-face and edge-edge rows.
#include "stages.cuh"

namespace ccd {

namespace {
size_t up(size_t x) { return scratch_up(x); }
}  // namespace

StageScratch stage_scratch_view(void *base, int64_t cap) {
  const size_t c = (size_t)cap;
  char *p = (char *)base;
  StageScratch sc;
  sc.cap = cap;
  sc.coef = (double *)p;
  p += up(kMaxSlots * 7 * c * sizeof(double));
  sc.span_l = (double *)p;
  p += up(kMaxSlots * 7 * c * sizeof(double));
  sc.span_u = (double *)p;
  p += up(kMaxSlots * 7 * c * sizeof(double));
  sc.roots = (double *)p;
  p += up(kMaxSlots * 6 * c * sizeof(double));
  sc.job_row = (int32_t *)p;
  p += up(kMaxSlots * c * sizeof(int32_t));
  sc.job_deg = (uint8_t *)p;
  p += up(kMaxSlots * c);
  sc.span_n = (uint8_t *)p;
  p += up(kMaxSlots * c);
  sc.queue = (unsigned *)p;
  p += up((kMaxSlots + 1) * sizeof(unsigned));
  sc.row_status = (uint32_t *)p;
  sc.jcap = 0;
  sc.wd = nullptr;
  sc.wi = nullptr;
  sc.wlist = nullptr;
  sc.wcount = nullptr;
  sc.tail = nullptr;
  sc.wave_steps = 0;
  sc.wave_min_rows = 0;
  sc.pool_budget = 0;
  sc.warp_finish = 1;
  sc.shift_after = 2;
  sc.pool_slots = stages::kWarpPool;
  sc.pool_slots_min = stages::kWarpPool;
  sc.pool_all = 0;
  sc.pool_phase_sync = 0;
  return sc;
}

size_t wave_scratch_bytes(int64_t cap) {
  const size_t j = (size_t)kMaxSlots * (size_t)cap;
  return up(jt::kDoubles * j * sizeof(double)) + up(jt::kInts * j * sizeof(int)) +
         up(2 * kWaveBins * j * sizeof(uint32_t)) + up((3 * kWaveBins + 2) * sizeof(unsigned)) +
         up(j * sizeof(uint32_t));
}

void attach_wave(StageScratch &sc, void *base) {
  const size_t j = (size_t)kMaxSlots * (size_t)sc.cap;
  char *p = (char *)base;
  sc.jcap = (int64_t)j;
  sc.wd = (double *)p;
  p += up(jt::kDoubles * j * sizeof(double));
  sc.wi = (int *)p;
  p += up(jt::kInts * j * sizeof(int));
  sc.wlist = (uint32_t *)p;
  p += up(2 * kWaveBins * j * sizeof(uint32_t));
  sc.wcount = (unsigned *)p;
  p += up((3 * kWaveBins + 2) * sizeof(unsigned));
  sc.tail = (uint32_t *)p;
  sc.wave_steps = kWaveSteps;
  sc.wave_min_rows = kWaveMinRows;
  sc.pool_budget = kPoolBudget;
}

namespace {
__global__ void all_rows(int64_t n, int32_t *list, BatchCounters *c) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) list[i] = (int32_t)i;
  if (i == 0) c->survivors = (unsigned long long)n;
}
}  // namespace

cudaError_t launch_all_rows(const PrimBatch &b, int32_t *list, cudaStream_t s) {
  if (b.n <= 0) return cudaSuccess;
  all_rows<<<(unsigned)((b.n + 255) / 256), 256, 0, s>>>(b.n, list, b.counters);
  return cudaGetLastError();
}

cudaError_t launch_stages(const PrimBatch &b, const int32_t *list, const StageScratch &sc, int num_sms,
                          cudaStream_t s, int *launches) {
  if (b.n <= 0) return cudaSuccess;
  if (b.kind == kVF) return stages::run<VFPolys>(b, list, sc, num_sms, s, launches);
  if (b.kind == kEE) return stages::run<EEPolys>(b, list, sc, num_sms, s, launches);
  return cudaErrorInvalidValue;
}

}  // namespace ccd
