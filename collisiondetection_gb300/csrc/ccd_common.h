// Shared definitions for the CTCD kernels.  Everything in csrc/*.h compiles
// both as CUDA device code (the product) and as plain host C++ (so the unit
// tests can check the device arithmetic against the oracle without a GPU).
//
// Build rule for every translation unit that includes these headers: no
// floating-point contraction (nvcc --fmad=false, g++ -ffp-contract=off).
// The reference's arithmetic is one IEEE rounding per operation; fused
// multiply-adds are only used where written explicitly as fma().
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define CCD_HD __host__ __device__ __forceinline__
#define CCD_HDI __host__ __device__
#define CCD_UNROLL _Pragma("unroll")
// One out-of-line copy of large routines keeps the kernels' instruction
// footprint small (the root finder and exp/log are called from many sites).
#define CCD_NOINLINE __host__ __device__ __noinline__ inline
#else
#include <cmath>
#define CCD_HD inline
#define CCD_HDI
#define CCD_UNROLL
#define CCD_NOINLINE __attribute__((noinline)) inline
#endif

namespace ccd {

// std::min / std::max with their exact argument semantics (the first argument
// is returned on ties and when the comparison involves NaN).
CCD_HD double smin(double a, double b) { return (b < a) ? b : a; }
CCD_HD double smax(double a, double b) { return (a < b) ? b : a; }

// Per-test status bits written next to each result.
enum : uint8_t {
  kStatusOk = 0,
  kStatusRootLimit = 1,  // root-bound iteration did not settle (non-finite coefficients)
};

// Primitive kinds; row widths are the reference's argument lists
// (include/CTCD.h:36-79): VF/EE 8 points, VE 6, VV 4 (start points, then end points).
enum Kind : int { kVF = 0, kEE = 1, kVE = 2, kVV = 3 };

}  // namespace ccd
