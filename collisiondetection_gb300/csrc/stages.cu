// Staged FP64 refinement (stages.cuh): scratch layout and the launchers for
// vertex-face and edge-edge rows.
#include "stages.cuh"

namespace ccd {

namespace {
constexpr size_t kAlign = 256;
size_t up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }
}  // namespace

size_t stage_scratch_bytes(int64_t cap) {
  const size_t c = (size_t)cap;
  return up(kMaxSlots * 7 * c * sizeof(double)) * 3 + up(kMaxSlots * 6 * c * sizeof(double)) +
         up(kMaxSlots * c * sizeof(int32_t)) +
         up(kMaxSlots * c) * 2 + up((kMaxSlots + 1) * sizeof(unsigned)) + up(c * sizeof(uint32_t));
}

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

cudaError_t launch_stages(const PrimBatch &b, const int32_t *list, const StageScratch &sc, int num_sms,
                          cudaStream_t s, int *launches) {
  if (b.n <= 0) return cudaSuccess;
  if (b.kind == kVF) return stages::run<VFPolys>(b, list, sc, num_sms, s, launches);
  if (b.kind == kEE) return stages::run<EEPolys>(b, list, sc, num_sms, s, launches);
  return cudaErrorInvalidValue;
}

}  // namespace ccd
