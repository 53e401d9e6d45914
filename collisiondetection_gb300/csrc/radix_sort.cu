// Stable LSD radix sort and exclusive scan (radix_sort.cuh).
#include "radix_sort.cuh"

namespace ccd {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;  // keys per block
constexpr int kWarps = kThreads / 32;
constexpr int kRun = kTile / kWarps;      // keys per warp run (contiguous)

size_t align_up(size_t x) { return (x + 255) / 256 * 256; }

// ------------------------------------------------------------------ scan
// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t &total) {
  __shared__ uint32_t warp_sums[kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kWarps ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kWarps) warp_sums[lane] = w;  // inclusive warp prefix
  }
  __syncthreads();
  total = warp_sums[kWarps - 1];
  const uint32_t before = warp > 0 ? warp_sums[warp - 1] : 0;
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(kThreads) scan_tiles(const uint32_t *in, uint32_t *out, int64_t n,
                                                       uint32_t *tile_sums) {
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
  uint32_t v[kItems];
  uint32_t sum = 0;
#pragma unroll
  for (int i = 0; i < kItems; i++) {
    v[i] = (base + i < n) ? in[base + i] : 0u;
    sum += v[i];
  }
  uint32_t total;
  uint32_t run = block_exclusive(sum, total);
#pragma unroll
  for (int i = 0; i < kItems; i++) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kThreads) add_offsets(uint32_t *out, int64_t n, const uint32_t *tile_offs) {
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
  const uint32_t add = tile_offs[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kItems; i++)
    if (base + i < n) out[base + i] += add;
}

__global__ void write_total(const uint32_t *scanned, const uint32_t *in, int64_t n, uint32_t *total) {
  *total = n > 0 ? scanned[n - 1] + in[n - 1] : 0u;
}

// ------------------------------------------------------------------ radix sort
__global__ void __launch_bounds__(kThreads) digit_histogram(const uint64_t *keys, int64_t n, int shift,
                                                            uint32_t *counts, int nblocks) {
  __shared__ uint32_t hist[256];
  hist[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kTile;
  for (int i = threadIdx.x; i < kTile; i += kThreads) {
    const int64_t k = base + i;
    if (k < n) atomicAdd(&hist[(keys[k] >> shift) & 255u], 1u);
  }
  __syncthreads();
  counts[(int64_t)threadIdx.x * nblocks + blockIdx.x] = hist[threadIdx.x];
}

__global__ void __launch_bounds__(kThreads) digit_scatter(const uint64_t *keys, const uint32_t *vals, uint64_t *okeys,
                                                          uint32_t *ovals, int64_t n, int shift,
                                                          const uint32_t *offsets, int nblocks) {
  __shared__ uint32_t warp_hist[kWarps][256];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  for (int i = threadIdx.x; i < kWarps * 256; i += kThreads) (&warp_hist[0][0])[i] = 0;
  __syncthreads();
  const int64_t run0 = (int64_t)blockIdx.x * kTile + (int64_t)warp * kRun;
  // Digit counts of this warp's run.
  for (int c = 0; c < kRun; c += 32) {
    const int64_t k = run0 + c + lane;
    if (k < n) atomicAdd(&warp_hist[warp][(keys[k] >> shift) & 255u], 1u);
  }
  __syncthreads();
  // Per digit: offsets of the warp runs inside the block, then the block's
  // global offset.
  {
    const int d = threadIdx.x;
    uint32_t run = offsets[(int64_t)d * nblocks + blockIdx.x];
    for (int w = 0; w < kWarps; w++) {
      const uint32_t c = warp_hist[w][d];
      warp_hist[w][d] = run;
      run += c;
    }
  }
  __syncthreads();
  // Stable scatter: runs in order, chunks of 32 in order, lanes in order.
  for (int c = 0; c < kRun; c += 32) {
    const int64_t k = run0 + c + lane;
    const bool valid = k < n;
    uint64_t key = valid ? keys[k] : 0;
    const unsigned d = valid ? (unsigned)((key >> shift) & 255u) : 256u + lane;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    uint32_t pos = 0;
    if (valid) pos = warp_hist[warp][d] + __popc(peers & lt);
    __syncwarp();
    if (valid && (peers & lt) == 0) warp_hist[warp][d] += __popc(peers);
    __syncwarp();
    if (valid) {
      okeys[pos] = key;
      if (vals) ovals[pos] = vals[k];
    }
  }
}

}  // namespace

size_t scan_temp_bytes(int64_t n) {
  size_t bytes = 0;
  int64_t m = n;
  while (true) {
    const int64_t tiles = (m + kTile - 1) / kTile;
    bytes += 2 * align_up((size_t)tiles * sizeof(uint32_t));
    if (tiles <= 1) break;
    m = tiles;
  }
  return bytes + 256;
}

static cudaError_t scan_rec(const uint32_t *in, uint32_t *out, int64_t n, char *temp, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t tiles = (n + kTile - 1) / kTile;
  uint32_t *sums = (uint32_t *)temp;
  uint32_t *offs = (uint32_t *)(temp + align_up((size_t)tiles * sizeof(uint32_t)));
  char *next = temp + 2 * align_up((size_t)tiles * sizeof(uint32_t));
  scan_tiles<<<(unsigned)tiles, kThreads, 0, s>>>(in, out, n, sums);
  if (tiles > 1) {
    cudaError_t e = scan_rec(sums, offs, tiles, next, s);
    if (e != cudaSuccess) return e;
    add_offsets<<<(unsigned)tiles, kThreads, 0, s>>>(out, n, offs);
  }
  return cudaGetLastError();
}

cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *total, void *temp,
                               size_t temp_bytes, cudaStream_t s) {
  if (temp_bytes < scan_temp_bytes(n)) return cudaErrorInvalidValue;
  if (total && n > 0 && in == out) return cudaErrorInvalidValue;  // the total needs the input
  cudaError_t e = scan_rec(in, out, n, (char *)temp, s);
  if (e != cudaSuccess) return e;
  if (total) {
    if (n > 0)
      write_total<<<1, 1, 0, s>>>(out, in, n, total);
    else
      e = cudaMemsetAsync(total, 0, sizeof(uint32_t), s);
  }
  return e != cudaSuccess ? e : cudaGetLastError();
}

size_t radix_sort_temp_bytes(int64_t n) {
  const int64_t nblocks = (n + kTile - 1) / kTile;
  const int64_t m = 256 * nblocks;
  return 2 * align_up((size_t)m * sizeof(uint32_t)) + scan_temp_bytes(m);
}

cudaError_t radix_sort_u64(uint64_t *keys, uint64_t *keys_alt, uint32_t *vals, uint32_t *vals_alt, int64_t n,
                           int begin_bit, int end_bit, void *temp, size_t temp_bytes, cudaStream_t s) {
  if (n <= 1) return cudaSuccess;
  if (n >= (int64_t)1 << 31 || temp_bytes < radix_sort_temp_bytes(n)) return cudaErrorInvalidValue;
  const int64_t nblocks = (n + kTile - 1) / kTile;
  const int64_t m = 256 * nblocks;
  uint32_t *counts = (uint32_t *)temp;
  uint32_t *offsets = (uint32_t *)((char *)temp + align_up((size_t)m * sizeof(uint32_t)));
  char *scan_tmp = (char *)temp + 2 * align_up((size_t)m * sizeof(uint32_t));
  uint64_t *src = keys, *dst = keys_alt;
  uint32_t *vsrc = vals, *vdst = vals_alt;
  int passes = 0;
  for (int shift = begin_bit; shift < end_bit; shift += 8, passes++) {
    digit_histogram<<<(unsigned)nblocks, kThreads, 0, s>>>(src, n, shift, counts, (int)nblocks);
    cudaError_t e = scan_rec(counts, offsets, m, scan_tmp, s);
    if (e != cudaSuccess) return e;
    digit_scatter<<<(unsigned)nblocks, kThreads, 0, s>>>(src, vsrc, dst, vdst, n, shift, offsets, (int)nblocks);
    uint64_t *t = src;
    src = dst;
    dst = t;
    uint32_t *tv = vsrc;
    vsrc = vdst;
    vdst = tv;
  }
  if (passes & 1) {
    cudaError_t e = cudaMemcpyAsync(keys, src, (size_t)n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
    if (vals) {
      e = cudaMemcpyAsync(vals, vsrc, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return e;
    }
  }
  return cudaGetLastError();
}

}  // namespace ccd
