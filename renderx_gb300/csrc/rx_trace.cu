// Closest-hit kernels (reference KDTree::intersect over a ray batch).
#include "rx_internal.h"
#include "rx_trace.cuh"

namespace rx {

// counters[0]: rays queued for the eager re-walk by the current launch, [1]: box
// tests decided by the exact test, [2]: rays re-walked (cumulative), [3]: errors
__global__ void __launch_bounds__(128) k_trace_closest(DevAccel A, const rx_ray* __restrict__ rays, uint32_t n,
                                                       int32_t* __restrict__ out_tid, float* __restrict__ out_dist,
                                                       uint32_t* __restrict__ eager_queue,
                                                       unsigned long long* __restrict__ counters) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned n_exact = 0;
  bool lazy_fail = false;
  if (i < n) {
    const float4* rp = reinterpret_cast<const float4*>(rays + i);
    float4 ro = __ldg(rp), rd = __ldg(rp + 1);
    F3 o = f3(ro), d = f3(rd);
    HitResult h = trace_ref_exact<false>(A, o, d, &n_exact);
    if (h.hit) {
      F3 inv = safe_inv(d);
      bool zd = (d.x == 0.0f) | (d.y == 0.0f) | (d.z == 0.0f);
      lazy_fail = !ref_visible(A, h.leaf, o, d, inv, zd, &n_exact);
    }
    if (lazy_fail) {
      unsigned long long slot = atomicAdd(&counters[0], 1ull);
      eager_queue[slot] = i;  // queue holds n entries: never overflows
    } else {
      out_tid[i] = h.hit ? h.tid : -1;
      out_dist[i] = h.hit ? h.t : -1.0f;
    }
  }
  // one atomic per warp for the diagnostics
  unsigned sum = n_exact;
  for (int s = 16; s > 0; s >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, s);
  if ((threadIdx.x & 31) == 0 && sum) atomicAdd(&counters[1], (unsigned long long)sum);
}

// Re-traces the queued rays checking visibility at every improvement.
__global__ void __launch_bounds__(128) k_trace_eager(DevAccel A, const rx_ray* __restrict__ rays,
                                                     int32_t* __restrict__ out_tid, float* __restrict__ out_dist,
                                                     const uint32_t* __restrict__ eager_queue,
                                                     unsigned long long* __restrict__ counters) {
  unsigned long long total = counters[0];
  if (blockIdx.x == 0 && threadIdx.x == 0 && total) atomicAdd(&counters[2], total);
  unsigned n_exact = 0;
  for (unsigned long long q = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; q < total;
       q += (unsigned long long)gridDim.x * blockDim.x) {
    uint32_t i = eager_queue[q];
    const float4* rp = reinterpret_cast<const float4*>(rays + i);
    float4 ro = __ldg(rp), rd = __ldg(rp + 1);
    HitResult h = trace_ref_exact<true>(A, f3(ro), f3(rd), &n_exact);
    out_tid[i] = h.hit ? h.tid : -1;
    out_dist[i] = h.hit ? h.t : -1.0f;
  }
  if (n_exact) atomicAdd(&counters[1], (unsigned long long)n_exact);
}

// The reference's own walk (KDTree.cpp:368-406) on the reference tree: every node whose
// box passes is entered, both children, no pruning; ties resolved exactly as there.
// ref node layout: a = (min.xyz, parent), b = (max.xyz, right child or ~leaf index).
__global__ void __launch_bounds__(128) k_trace_reforder(DevAccel A, const rx_ray* __restrict__ rays, uint32_t n,
                                                        int32_t* __restrict__ out_tid, float* __restrict__ out_dist,
                                                        unsigned long long* __restrict__ counters) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4* rp = reinterpret_cast<const float4*>(rays + i);
  float4 ro = __ldg(rp), rd = __ldg(rp + 1);
  F3 o = f3(ro), d = f3(rd);
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  bool have = false;
  float bt = -1.0f;
  int32_t btid = -1;
  uint32_t bleaf = 0;
  while (sp > 0) {
    int node = stack[--sp];
    float4 a = __ldg(&A.ref[2 * node]), b = __ldg(&A.ref[2 * node + 1]);
    if (!box_exact(f3(a), f3(b), o, d)) continue;
    int r = __float_as_int(b.w);
    if (r >= 0) {
      if (sp + 2 > 128) { atomicAdd(&counters[3], 1ull); break; }
      stack[sp++] = r;         // right after left: left is popped first (DFS order)
      stack[sp++] = node + 1;  // pre-order: the left child follows its parent
      continue;
    }
    uint32_t leaf = (uint32_t)~r;
    uint32_t beg = A.ref_leaf_range[2 * leaf], end = A.ref_leaf_range[2 * leaf + 1];
    for (uint32_t k = beg; k < end; k++) {
      const float4* tp = A.ref_tris + 3 * (size_t)k;
      float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
      float t;
      if (tri_exact(f3(v0), f3(v1), f3(v2), o, d, t)) {
        // leaves come in DFS order: a later leaf wins ties, inside a leaf the first
        if (!have || t < bt || (t == bt && leaf != bleaf)) {
          have = true;
          bt = t;
          bleaf = leaf;
          btid = __float_as_int(v0.w);
        }
      }
    }
  }
  out_tid[i] = have ? btid : -1;
  out_dist[i] = have ? bt : -1.0f;
}

cudaError_t launch_trace_closest(const DevAccel& A, const rx_ray* rays, uint32_t n, int32_t* tid, float* dist,
                                 uint32_t* queue, unsigned long long* counters, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  cudaMemsetAsync(counters, 0, sizeof(unsigned long long), s);  // queue length
  k_trace_closest<<<(n + 127) / 128, 128, 0, s>>>(A, rays, n, tid, dist, queue, counters);
  k_trace_eager<<<152, 128, 0, s>>>(A, rays, tid, dist, queue, counters);
  return cudaGetLastError();
}

cudaError_t launch_trace_reforder(const DevAccel& A, const rx_ray* rays, uint32_t n, int32_t* tid, float* dist,
                                  unsigned long long* counters, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_trace_reforder<<<(n + 127) / 128, 128, 0, s>>>(A, rays, n, tid, dist, counters);
  return cudaGetLastError();
}

}  // namespace rx
