// Stable LSD radix sort of 64-bit keys (optionally with 32-bit values) and a
// device-wide exclusive scan, for the broad phase (Morton order, stencil
// deduplication).  8-bit digits; each pass is histogram -> scan -> stable
// scatter.  Stability inside a tile: every warp scans a contiguous run of the
// tile in order and ranks equal digits with __match_any_sync.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ccd {

// Temporary storage needed by radix_sort_u64 for n keys.
size_t radix_sort_temp_bytes(int64_t n);

// Sorts keys (and values, when non-null) ascending by the bits
// [begin_bit, end_bit).  keys_alt / vals_alt are scratch of the same size;
// the sorted data ends up in keys / vals.
cudaError_t radix_sort_u64(uint64_t *keys, uint64_t *keys_alt, uint32_t *vals, uint32_t *vals_alt, int64_t n,
                           int begin_bit, int end_bit, void *temp, size_t temp_bytes, cudaStream_t s);

// Exclusive prefix sum of n uint32 counts into out (out may alias in); the
// total is written to *total (device pointer) when non-null.
size_t scan_temp_bytes(int64_t n);
cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, int64_t n, uint32_t *total, void *temp,
                               size_t temp_bytes, cudaStream_t s);

}  // namespace ccd
