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

// ---- exclusive prefix sums over n counters (any n): block scans of 1024 entries, a
// carry scan of the block sums in one block, then the block offsets. start may alias
// count (each thread reads its entry before the block writes). Internal linkage: every
// translation unit that includes this header launches its own instantiations.
namespace {
template <class T>
__global__ void k_scan_blocks(const T* count, T* start, T* block_sum, unsigned n) {
  __shared__ T s[1024];
  unsigned i = blockIdx.x * 1024 + threadIdx.x;
  T v = i < n ? count[i] : T(0);
  s[threadIdx.x] = v;
  __syncthreads();
  for (unsigned off = 1; off < 1024; off <<= 1) {
    T t = threadIdx.x >= off ? s[threadIdx.x - off] : T(0);
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) start[i] = s[threadIdx.x] - v;
  if (threadIdx.x == 1023) block_sum[blockIdx.x] = s[1023];
}
template <class T>
__global__ void k_scan_sums(T* block_sum, unsigned nb) {
  // single block, sequential carry over chunks of 1024
  __shared__ T s[1024];
  T carry = 0;
  for (unsigned base = 0; base < nb; base += 1024) {
    unsigned i = base + threadIdx.x;
    T v = i < nb ? block_sum[i] : T(0);
    s[threadIdx.x] = v;
    __syncthreads();
    for (unsigned off = 1; off < 1024; off <<= 1) {
      T t = threadIdx.x >= off ? s[threadIdx.x - off] : T(0);
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) block_sum[i] = carry + s[threadIdx.x] - v;
    __syncthreads();
    carry += s[1023];
    __syncthreads();
  }
}
template <class T>
__global__ void k_scan_add(T* start, const T* block_sum, unsigned n, T* cursor) {
  unsigned i = blockIdx.x * 1024 + threadIdx.x;
  if (i < n) {
    start[i] += block_sum[blockIdx.x];
    if (cursor) cursor[i] = start[i];
  }
}

}  // namespace

// Exclusive prefix sum of the kRayBins counters, in place, with scratch for the block
// sums (kRayBins / 1024 entries).
static inline void scan_bins(uint32_t* hist, uint32_t* block_sums, cudaStream_t s) {
  constexpr unsigned nb = kRayBins / 1024;
  k_scan_blocks<uint32_t><<<nb, 1024, 0, s>>>(hist, hist, block_sums, kRayBins);
  k_scan_sums<uint32_t><<<1, 1024, 0, s>>>(block_sums, nb);
  k_scan_add<uint32_t><<<nb, 1024, 0, s>>>(hist, block_sums, kRayBins, nullptr);
}
// order[cursor[keys[i]]++] = i for the n rays (n = *count when count is non-null).
__global__ void k_ray_scatter(const uint32_t* __restrict__ keys, uint32_t n_host, const unsigned* count,
                              uint32_t* __restrict__ cursor, uint32_t* __restrict__ order);

}  // namespace rx
