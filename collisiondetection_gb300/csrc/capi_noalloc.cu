// Allocation-free batch entry point (include/ccd_gb300.h,
// ccd_prim_batch_device_noalloc).  No counterpart in the reference.
//
// Why it exists: cudaMalloc and cudaFree synchronise the whole device, and
// they can fail outright once a host framework's caching allocator has
// reserved most of the GPU's memory up front.  A caller in the middle of a
// time step -- a simulation loop whose other streams must not stall, or a host
// that owns all device memory through its own pool -- therefore cannot let a
// collision query allocate.  This entry point runs the same FP32 rejection and
// staged FP64 refinement kernels as ccd_prim_batch_device with
// CCD_PATH_CULL_REFINE, but takes every byte of scratch from one fixed
// file-scope device array instead of a context's growable buffers.
//
// Limits and rules:
//   * at most CCD_NOALLOC_MAX_ROWS rows per call; larger n is rejected with
//     CCD_ERR_INVALID_ARGUMENT before anything is enqueued;
//   * the scratch is one region per device, so calls whose device work can
//     overlap in time (different streams, or several host threads) race on
//     it and corrupt each other's results: issue them on one stream or
//     serialise them;
//   * the first call on each device does the setup (looks up the scratch
//     address and the SM count with that device current); make that first
//     call before any stream capture that should contain later calls;
//   * the only scratch that must start at zero is the batch counter block,
//     which each call clears on the caller's stream before its kernels (the
//     staged refinement clears its own job queues per tile; every other
//     scratch array is written before it is read).
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/ccd_gb300.h"
#include "narrow.cuh"
#include "stages.cuh"

namespace {

// Survivor rows per staged-refinement tile (the tile loop covers up to
// CCD_NOALLOC_MAX_ROWS survivors in 8 tiles).
constexpr int64_t kTileRows = 8192;
constexpr size_t kAlign = 256;

constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Layout: [batch counters | survivor list (max rows) | staged-refinement tile].
constexpr size_t kCountersOff = 0;
constexpr size_t kSurvOff = align_up(sizeof(ccd::BatchCounters));
constexpr size_t kStageOff = kSurvOff + align_up((size_t)CCD_NOALLOC_MAX_ROWS * sizeof(int32_t));
constexpr size_t kStageBytes = ccd::stage_scratch_bytes(kTileRows);
constexpr size_t kScratchBytes = kStageOff + kStageBytes;  // about 9.4 MB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;

struct DeviceSetup {
  bool ready = false;
  unsigned char *scratch = nullptr;
  int num_sms = 0;
};

std::mutex g_setup_mutex;
DeviceSetup g_setup[kMaxDevices];

// Looks up the scratch address and SM count of the current device once.
int setup_current_device(DeviceSetup *out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CCD_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return CCD_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceSetup &d = g_setup[dev];
  if (!d.ready) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return CCD_ERR_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
      return CCD_ERR_CUDA;
    d.scratch = (unsigned char *)p;
    d.num_sms = sms;
    d.ready = true;
  }
  *out = d;
  return CCD_OK;
}

}  // namespace

extern "C" int ccd_prim_batch_device_noalloc(int kind, int64_t n, const double *rows, const double *eta,
                                             int64_t eta_count, uint8_t *hit, double *t, void *stream) {
  if (kind < CCD_VERTEX_FACE || kind > CCD_VERTEX_VERTEX) return CCD_ERR_INVALID_ARGUMENT;
  if (n < 0 || n > CCD_NOALLOC_MAX_ROWS) return CCD_ERR_INVALID_ARGUMENT;
  if (n == 0) return CCD_OK;
  if (!rows || !eta || !hit || !t) return CCD_ERR_INVALID_ARGUMENT;
  if (eta_count != 1 && eta_count != n) return CCD_ERR_INVALID_ARGUMENT;
  DeviceSetup d;
  const int rc = setup_current_device(&d);
  if (rc != CCD_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  ccd::BatchCounters *counters = (ccd::BatchCounters *)(d.scratch + kCountersOff);
  int32_t *surv = (int32_t *)(d.scratch + kSurvOff);
  const ccd::StageScratch stage = ccd::stage_scratch_view(d.scratch + kStageOff, kTileRows);
  const ccd::PrimBatch b{kind, n, rows, eta, eta_count == n && n != 1, hit, t, nullptr, counters};
  if (cudaMemsetAsync(counters, 0, sizeof(ccd::BatchCounters), s) != cudaSuccess) return CCD_ERR_CUDA;
  // The kernels of the batch entry points' cull + refine path: vertex-vertex
  // rows (one quadratic) in FP64 directly, vertex-edge survivors by one FP64
  // pass over the survivor list, vertex-face and edge-edge survivors by the
  // staged refinement in tiles of kTileRows.
  cudaError_t e;
  if (kind == CCD_VERTEX_VERTEX) {
    e = ccd::launch_prims_fp64(b, d.num_sms, s);
  } else if (kind == CCD_VERTEX_EDGE) {
    e = ccd::launch_prims_cull(b, surv, d.num_sms, s);
    if (e == cudaSuccess) e = ccd::launch_prims_fp64_list(b, surv, d.num_sms, s);
  } else {
    e = ccd::launch_prims_cull(b, surv, d.num_sms, s);
    int launches = 0;
    if (e == cudaSuccess) e = ccd::launch_stages(b, surv, stage, d.num_sms, s, &launches);
  }
  return e == cudaSuccess ? CCD_OK : CCD_ERR_CUDA;
}
