// Ray binning: a counting sort of rays by (origin cell, direction bin) so that a warp's
// traversals start close together and head the same way. Key: Morton code of the
// origin's cell on a 2^c per axis grid over the scene bounds (3c bits), then a
// direction bin (dir_key). The closest-hit batch takes c = 4 and the octahedral map on a
// 16 x 16 grid (2^20 bins); ray_key's defaults, c = 4 with 4 levels per direction
// component (kRayBins = 2^18 bins), serve the path tracer and VCM's queries.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "rx_internal.h"

namespace rx {

__device__ __forceinline__ uint32_t spread3(uint32_t v) {  // 5 bits -> every third bit
  v &= 31u;
  return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6) | ((v & 16u) << 8);
}

__device__ __forceinline__ uint32_t spread2(uint32_t v) {  // 6 bits -> every second bit
  v &= 63u;
  v = (v | (v << 2)) & 0x333u;
  return (v | (v << 1)) & 0x555u;
}

// The direction bin. dir_map 0: each component quantised to 2^dbits levels (3 dbits
// bits); 1: the octahedral map of the direction (the unit sphere folded onto a square)
// on a 2^dbits x 2^dbits grid in Morton order (2 dbits bits), bins of near-equal solid
// angle with neighbouring bins near in direction.
__device__ __forceinline__ uint32_t dir_key(float4 d, int dbits, int dir_map) {
  const float levels = (float)(1 << dbits);
  if (dir_map == 0) {
    float q[3] = {d.x, d.y, d.z};
    uint32_t dir[3];
#pragma unroll
    for (int k = 0; k < 3; k++) dir[k] = (uint32_t)fminf(fmaxf((q[k] + 1.0f) * (0.5f * levels), 0.0f), levels - 1.0f);
    return (dir[0] << (2 * dbits)) | (dir[1] << dbits) | dir[2];
  }
  const float s = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
  float u = s > 0.0f ? d.x / s : 0.0f, v = s > 0.0f ? d.y / s : 0.0f;
  if (d.z < 0.0f) {
    const float fu = (1.0f - fabsf(v)) * (u < 0.0f ? -1.0f : 1.0f), fv = (1.0f - fabsf(u)) * (v < 0.0f ? -1.0f : 1.0f);
    u = fu;
    v = fv;
  }
  const uint32_t iu = (uint32_t)fminf(fmaxf((u + 1.0f) * (0.5f * levels), 0.0f), levels - 1.0f);
  const uint32_t iv = (uint32_t)fminf(fmaxf((v + 1.0f) * (0.5f * levels), 0.0f), levels - 1.0f);
  return spread2(iu) | (spread2(iv) << 1);
}

// The key: the origin cell's Morton code, then the direction bin. cbits <= 5; dir_map
// 0: dbits <= 3, 3 (cbits + dbits) <= 21; 1: dbits <= 6, 3 cbits + 2 dbits <= 21.
__device__ __forceinline__ uint32_t ray_key(const float (&lo)[3], const float (&hi)[3], float4 o, float4 d,
                                            int cbits = 4, int dbits = 2, int dir_map = 0) {
  const float cells = (float)(1 << cbits);
  float p[3] = {o.x, o.y, o.z};
  uint32_t cell[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float t = (p[k] - lo[k]) / fmaxf(hi[k] - lo[k], 1e-20f) * cells;
    cell[k] = (uint32_t)fminf(fmaxf(t, 0.0f), cells - 1.0f);
  }
  uint32_t morton = spread3(cell[0]) | (spread3(cell[1]) << 1) | (spread3(cell[2]) << 2);
  return (morton << ((dir_map ? 2 : 3) * dbits)) | dir_key(d, dbits, dir_map);
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

// Exclusive prefix sum of `bins` counters (a multiple of 1024), in place, with scratch
// for the block sums (bins / 1024 entries).
static inline void scan_bins(uint32_t* hist, uint32_t* block_sums, cudaStream_t s, uint32_t bins = kRayBins) {
  const unsigned nb = bins / 1024;
  k_scan_blocks<uint32_t><<<nb, 1024, 0, s>>>(hist, hist, block_sums, bins);
  k_scan_sums<uint32_t><<<1, 1024, 0, s>>>(block_sums, nb);
  k_scan_add<uint32_t><<<nb, 1024, 0, s>>>(hist, block_sums, bins, nullptr);
}
// order[cursor[keys[i]]++] = i for the n rays (n = *count when count is non-null).
__global__ void k_ray_scatter(const uint32_t* __restrict__ keys, uint32_t n_host, const unsigned* count,
                              uint32_t* __restrict__ cursor, uint32_t* __restrict__ order);

}  // namespace rx
