// common.cuh — device utilities shared by the build, traversal and shading
// kernels: error reporting, order-preserving float<->uint encodings for
// atomic min/max, scans.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "geom.cuh"

namespace wpbr {

// Device error word bits (read and cleared by wpbr_check_device_errors).
enum : uint32_t {
  kErrStackOverflow = 1u << 0,  // traversal stack exhausted
  kErrLoopLimit = 1u << 1,      // bounded loop hit its iteration cap
  kErrBuild = 1u << 2           // build invariant violated
};

// Monotonic float <-> uint map: a < b  <=>  enc(a) < enc(b) (for non-NaN).
__device__ __forceinline__ uint32_t fenc(float f) {
  uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fdec(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}
WPBR_HD uint32_t fenc_h(float f) {
  uint32_t u = f2u(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;  // 2048 elements per block

inline unsigned div_up(uint64_t a, uint64_t b) { return (unsigned)((a + b - 1) / b); }

// Grid for a persistent kernel: resident blocks per SM times the SM count.
inline unsigned persistent_grid(const void* kernel, int block = 128) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, 0);
  if (per_sm < 1) per_sm = 1;
  if (sms < 1) sms = 1;
  return (unsigned)(sms * per_sm);
}

}  // namespace wpbr
