// Ray binning: a counting sort of rays by (origin cell, direction bin) so that a warp's
// traversals start close together and head the same way. Key: Morton code of the
// origin's cell on a 16^3 grid over the scene bounds (12 bits), then the direction
// quantised to 4 levels per axis (6 bits): kRayBins = 2^18 bins.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "rx_internal.h"

namespace rx {

__device__ __forceinline__ uint32_t spread3(uint32_t v) {  // 4 bits -> every third bit
  v &= 15u;
  return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6);
}

__device__ __forceinline__ uint32_t ray_key(const float (&lo)[3], const float (&hi)[3], float4 o, float4 d) {
  float p[3] = {o.x, o.y, o.z}, q[3] = {d.x, d.y, d.z};
  uint32_t cell[3], dir[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float t = (p[k] - lo[k]) / fmaxf(hi[k] - lo[k], 1e-20f) * 16.0f;
    cell[k] = (uint32_t)fminf(fmaxf(t, 0.0f), 15.0f);
    dir[k] = (uint32_t)fminf(fmaxf((q[k] + 1.0f) * 2.0f, 0.0f), 3.0f);
  }
  uint32_t morton = spread3(cell[0]) | (spread3(cell[1]) << 1) | (spread3(cell[2]) << 2);
  return (morton << 6) | (dir[0] << 4) | (dir[1] << 2) | dir[2];
}

// Exclusive prefix sum of the kRayBins counters, in place (one block of 1024 threads).
__global__ void k_scan_bins(uint32_t* hist);
// order[cursor[keys[i]]++] = i for the n rays (n = *count when count is non-null).
__global__ void k_ray_scatter(const uint32_t* __restrict__ keys, uint32_t n_host, const unsigned* count,
                              uint32_t* __restrict__ cursor, uint32_t* __restrict__ order);

}  // namespace rx
