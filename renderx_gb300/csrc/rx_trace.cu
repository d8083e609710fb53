// Closest-hit kernels (reference KDTree::intersect over a ray batch).
#include "rx_internal.h"
#include "rx_bin.cuh"
#include "rx_trace.cuh"
#include "rx_accel.h"
#include "rx_walk.cuh"

namespace rx {

// counters[0]: rays queued for the eager re-walk by the current launch, [1]: box
// tests decided by the exact test, [2]: rays re-walked (cumulative), [3]: errors
constexpr uint32_t kNoLeaf = 0xffffffffu;

// Reference visibility of each ray's winner (KDTree.cpp:34-52 on every box of the
// winner's root path), one warp per ray and one root-path box per lane; the boxes of
// the reference tree are few and stay in cache. Rays whose winner the reference cannot
// see go to the eager queue.
__global__ void __launch_bounds__(128) k_check_visible(DevAccel A, const rx_ray* __restrict__ rays, uint32_t n,
                                                       const uint32_t* __restrict__ hit_leaf,
                                                       uint32_t* __restrict__ eager_queue,
                                                       unsigned long long* __restrict__ counters) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  unsigned n_exact = 0;
  for (uint32_t i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    uint32_t leaf = __ldg(&hit_leaf[i]);
    if (leaf == kNoLeaf) continue;
    const float4* rp = reinterpret_cast<const float4*>(rays + i);
    F3 o = f3(__ldg(rp)), d = f3(__ldg(rp + 1));
    F3 inv = safe_inv(d);
    const ClearMargins mg = clear_margins(o, d);
    bool zd = (d.x == 0.0f) | (d.y == 0.0f) | (d.z == 0.0f);
    uint32_t b = __ldg(&A.anc_range[2 * leaf]), e = __ldg(&A.anc_range[2 * leaf + 1]);
    bool ok = true;
    for (uint32_t base = b; base < e; base += 32) {
      uint32_t k = base + lane;
      bool pass = true;
      if (k < e) {
        int node = __ldg(&A.anc_nodes[k]);
        float4 lo = __ldg(&A.ref[2 * node]), hi = __ldg(&A.ref[2 * node + 1]);
        if (zd || !box_clear_pass(f3(lo), f3(hi), o, d, inv, mg)) {
          n_exact++;
          pass = box_exact(f3(lo), f3(hi), o, d);
        }
      }
      ok = __all_sync(FULL, pass) && ok;
    }
    if (!ok && lane == 0) {
      unsigned long long slot = atomicAdd(&counters[0], 1ull);
      eager_queue[slot] = i;  // the queue holds n entries: never overflows
    }
  }
  unsigned sum = n_exact;
  for (int s2 = 16; s2 > 0; s2 >>= 1) sum += __shfl_xor_sync(FULL, sum, s2);
  if (lane == 0 && sum) atomicAdd(&counters[1], (unsigned long long)sum);
}

// The closest-hit batch's lanes for walk_persistent: ray `order[r]` (binned order) or r,
// the reference's exact triangle test and tie rule (closest distance, then the larger
// reference leaf, then the earlier position), pruning at best + prune_rel (1 + best); the
// answer goes to the slot record (binned order; the check scatters it) or to the outputs.
struct HitLane {
  const DevAccel& A;
  const rx_ray* __restrict__ rays;
  uint32_t n;
  const uint32_t* __restrict__ order;
  int32_t* __restrict__ out_tid;
  float* __restrict__ out_dist;
  uint32_t* __restrict__ hit_leaf;
  int4* __restrict__ slot_rec;
  const float4* bvh;
  uint32_t ray = 0, slot = 0;
  float tlimit = INFINITY;
  HitResult best{-1, -1.0f, 0u, 0u, false};

  __device__ bool begin(uint32_t r, F3& o, F3& d) {
    if (r >= n) return false;
    slot = r;
    ray = order ? __ldg(&order[r]) : r;
    const float4* rp = reinterpret_cast<const float4*>(rays + ray);
    o = f3(__ldg(rp));
    d = f3(__ldg(rp + 1));
    tlimit = INFINITY;
    best = {-1, -1.0f, 0u, 0u, false};
    return true;
  }
  __device__ const float4* nodes() const { return bvh; }
  __device__ float limit() const { return tlimit; }
  __device__ void leaf(int first, int count, F3 o, F3 d) {
    for (int k = 0; k < count; k++) {
      const float4* tp = A.tris + 3 * (size_t)(first + k);
      float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
      float t;
      if (tri_exact_n(f3(v0), f3(v1), f3(v2), A.tri_nrm + first + k, o, d, t)) {
        uint32_t lf = __float_as_uint(v1.w), pos = __float_as_uint(v2.w);
        if (!best.hit || t < best.t || (t == best.t && (lf > best.leaf || (lf == best.leaf && pos < best.pos)))) {
          best = {__float_as_int(v0.w), t, lf, pos, true};
          tlimit = t + A.prune_rel * (1.0f + t);
        }
      }
    }
  }
  __device__ void end() {
    if (slot_rec) {  // one 16-byte record by binned slot; the check scatters it to ray order
      slot_rec[slot] = make_int4(best.hit ? best.tid : -1, __float_as_int(best.hit ? best.t : -1.0f),
                                 (int)(best.hit ? best.leaf : kNoLeaf), 0);
    } else {
      out_tid[ray] = best.hit ? best.tid : -1;
      out_dist[ray] = best.hit ? best.t : -1.0f;
      hit_leaf[ray] = best.hit ? best.leaf : kNoLeaf;
    }
  }
};

template <int W, int kShort, int kStack>
__device__ __forceinline__ void walk_wide(const DevAccel& A, const float4* __restrict__ nodes,
                                          const rx_ray* __restrict__ rays, uint32_t n,
                                          const uint32_t* __restrict__ order, int32_t* __restrict__ out_tid,
                                          float* __restrict__ out_dist, uint32_t* __restrict__ hit_leaf,
                                          int4* __restrict__ slot_rec, unsigned long long* __restrict__ counters) {
  HitLane L{A, rays, n, order, out_tid, out_dist, hit_leaf, slot_rec, nodes};
  walk_persistent<W, kShort, kStack>(L, counters + 4);
}

// 4-wide walk: 128-byte nodes; at most 3 stack entries per level of a tree shallower
// than 22 levels. At most 64 registers, so that eight blocks (32 warps) stay resident per
// SM: 2% faster than the 68 registers the compiler picks unbounded (seven blocks), on
// the 2^24-ray batch over 4.1 M triangles; tighter bounds spill the stack and lose.
template <int kShort>
__global__ void __launch_bounds__(128, 8) k_trace_persistent4(DevAccel A, const rx_ray* __restrict__ rays, uint32_t n,
                                                           const uint32_t* __restrict__ order,
                                                           int32_t* __restrict__ out_tid,
                                                           float* __restrict__ out_dist,
                                                           uint32_t* __restrict__ hit_leaf,
                                                           int4* __restrict__ slot_rec,
                                                           unsigned long long* __restrict__ counters) {
  walk_wide<4, kShort, 64>(A, A.bvh4, rays, n, order, out_tid, out_dist, hit_leaf, slot_rec, counters);
}

// 8-wide walk: 256-byte nodes; at most 7 stack entries per level of a tree shallower
// than 12 levels.
template <int kShort>
__global__ void __launch_bounds__(128) k_trace_persistent8(DevAccel A, const rx_ray* __restrict__ rays, uint32_t n,
                                                           const uint32_t* __restrict__ order,
                                                           int32_t* __restrict__ out_tid,
                                                           float* __restrict__ out_dist,
                                                           uint32_t* __restrict__ hit_leaf,
                                                           int4* __restrict__ slot_rec,
                                                           unsigned long long* __restrict__ counters) {
  walk_wide<8, kShort, 80>(A, A.bvh8, rays, n, order, out_tid, out_dist, hit_leaf, slot_rec, counters);
}

// The same check with one thread per ray: each thread walks its winner's ancestor list
// (four boxes per step); the lists and boxes of the reference tree are a few hundred KB
// and stay in L1/L2. Rays whose winner fails go to the eager queue (warp-aggregated).
__global__ void __launch_bounds__(128) k_check_visible_thread(DevAccel A, const rx_ray* __restrict__ rays,
                                                              uint32_t n, const uint32_t* __restrict__ order,
                                                              const uint32_t* __restrict__ hit_leaf,
                                                              const int4* __restrict__ slot_rec,
                                                              int32_t* __restrict__ out_tid,
                                                              float* __restrict__ out_dist,
                                                              uint32_t* __restrict__ eager_queue,
                                                              unsigned long long* __restrict__ counters) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t iters = (n + stride - 1) / stride;
  unsigned n_exact = 0;
  for (uint32_t it = 0; it < iters; it++) {
    uint32_t j = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t i = j < n && order ? __ldg(&order[j]) : j;  // binned order: a warp checks nearby leaves
    bool fail = false;
    if (j < n) {
      // slot_rec: the walk left its answer by binned slot; this is where it reaches ray
      // order (a rejected winner is re-walked after, overwriting it)
      uint32_t leaf;
      if (slot_rec) {
        const int4 rec = __ldg(slot_rec + j);
        out_tid[i] = rec.x;
        out_dist[i] = __int_as_float(rec.y);
        leaf = (uint32_t)rec.z;
      } else {
        leaf = __ldg(&hit_leaf[i]);
      }
      if (leaf != kNoLeaf) {
        const float4* rp = reinterpret_cast<const float4*>(rays + i);
        F3 o = f3(__ldg(rp)), d = f3(__ldg(rp + 1));
        bool zd = (d.x == 0.0f) | (d.y == 0.0f) | (d.z == 0.0f);
        fail = !ref_visible(A, leaf, o, d, safe_inv(d), zd, &n_exact);
      }
    }
    unsigned m = __ballot_sync(FULL, fail);
    if (m) {
      unsigned long long base = 0;
      int leader = __ffs(m) - 1;
      if (lane == leader) base = atomicAdd(&counters[0], (unsigned long long)__popc(m));
      base = __shfl_sync(FULL, base, leader);
      if (fail) eager_queue[base + __popc(m & ((1u << lane) - 1))] = i;  // at most n entries
    }
  }
  unsigned sum = n_exact;
  for (int s2 = 16; s2 > 0; s2 >>= 1) sum += __shfl_xor_sync(FULL, sum, s2);
  if (lane == 0 && sum) atomicAdd(&counters[1], (unsigned long long)sum);
}

// One thread per ray. Writes the winner and its reference leaf; k_check_visible then
// confirms the winner is visible to the reference.
__global__ void __launch_bounds__(128) k_trace_closest(DevAccel A, const rx_ray* __restrict__ rays, uint32_t n,
                                                       int32_t* __restrict__ out_tid, float* __restrict__ out_dist,
                                                       uint32_t* __restrict__ hit_leaf,
                                                       unsigned long long* __restrict__ counters) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  unsigned n_exact = 0;
  F3 o{0, 0, 0}, d{0, 0, 1};
  HitResult h{-1, -1.0f, 0u, 0u, false};
  if (i < n) {
    const float4* rp = reinterpret_cast<const float4*>(rays + i);
    float4 ro = __ldg(rp), rd = __ldg(rp + 1);
    o = f3(ro);
    d = f3(rd);
    h = trace_ref_exact<false>(A, o, d, &n_exact);
  }
  if (i < n) {
    out_tid[i] = h.hit ? h.tid : -1;
    out_dist[i] = h.hit ? h.t : -1.0f;
    hit_leaf[i] = h.hit ? h.leaf : kNoLeaf;
  }
  // one atomic per warp for the diagnostics
  unsigned sum = n_exact;
  for (int s = 16; s > 0; s >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, s);
  if (lane == 0 && sum) atomicAdd(&counters[1], (unsigned long long)sum);
}

// Persistent variant: warps stay resident and refill lanes whose ray has finished with
// the next rays of the batch (one atomic per warp and refill), so a warp never idles
// behind its longest ray. Each round walks inner nodes until the lane holds a leaf
// (SPEC: keeps walking with the leaf postponed until every lane of the warp holds one),
// then tests that leaf's triangles; finished lanes are checked for reference
// visibility together. counters[4] is the batch cursor.
template <bool SPEC, int kStack>
__global__ void __launch_bounds__(128) k_trace_persistent(DevAccel A, const rx_ray* __restrict__ rays, uint32_t n,
                                                          const uint32_t* __restrict__ order,
                                                          int32_t* __restrict__ out_tid,
                                                          float* __restrict__ out_dist,
                                                          uint32_t* __restrict__ hit_leaf,
                                                           int4* __restrict__ slot_rec,
                                                          unsigned long long* __restrict__ counters) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int DONE = INT_MIN;
  const int lane = threadIdx.x & 31;
  unsigned long long* cursor = counters + 4;
  bool active = false, exhausted = false;
  uint32_t ray = 0, slot = 0;
  F3 o{}, d{}, inv{}, ood{};
  float tlimit = INFINITY;
  HitResult best{-1, -1.0f, 0u, 0u, false};
  int stack_ref[kStack];
  float stack_tn[kStack];
  int sp = 0, cur = DONE, cnt = 0;
  unsigned n_exact = 0;

  auto pop = [&]() {
    while (sp > 0) {
      sp--;
      if (stack_tn[sp] <= tlimit) {
        int r = stack_ref[sp];
        if (r < 0) {
          int packed = ~r;
          cnt = (packed & 7) + 1;
          return ~(packed >> 3);
        }
        return r;
      }
    }
    return DONE;
  };

  while (true) {
    unsigned want = __ballot_sync(FULL, !active && !exhausted);
    if (want) {
      int leader = __ffs(want) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(cursor, (unsigned long long)__popc(want));
      base = __shfl_sync(FULL, base, leader);
      if (!active && !exhausted) {
        unsigned long long r = base + __popc(want & ((1u << lane) - 1));
        if (r < n) {
          slot = (uint32_t)r;
          ray = order ? __ldg(&order[r]) : (uint32_t)r;
          const float4* rp = reinterpret_cast<const float4*>(rays + ray);
          float4 ro = __ldg(rp), rd = __ldg(rp + 1);
          o = f3(ro);
          d = f3(rd);
          inv = safe_inv(d);
          ood = {o.x * inv.x, o.y * inv.y, o.z * inv.z};
          tlimit = INFINITY;
          best = {-1, -1.0f, 0u, 0u, false};
          sp = 0;
          cur = 0;
          cnt = 0;
          active = true;
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(FULL, active)) break;

    if (active) {
      int pl = DONE, pcnt = 0;  // postponed leaf
      while (true) {
        if (cur >= 0) {
          const float4* np = A.bvh + 4 * (size_t)cur;
          float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2);
          int4 n3 = __ldg(reinterpret_cast<const int4*>(np + 3));
          float a0 = fmaf(n0.x, inv.x, -ood.x), b0 = fmaf(n0.y, inv.x, -ood.x);
          float a1 = fmaf(n0.z, inv.y, -ood.y), b1 = fmaf(n0.w, inv.y, -ood.y);
          float a2 = fmaf(n2.x, inv.z, -ood.z), b2 = fmaf(n2.y, inv.z, -ood.z);
          float tn0 = fmaxf(fmaxf(fminf(a0, b0), fminf(a1, b1)), fmaxf(fminf(a2, b2), 0.0f));
          float tf0 = fminf(fminf(fmaxf(a0, b0), fmaxf(a1, b1)), fminf(fmaxf(a2, b2), tlimit));
          float c0 = fmaf(n1.x, inv.x, -ood.x), d0 = fmaf(n1.y, inv.x, -ood.x);
          float c1 = fmaf(n1.z, inv.y, -ood.y), d1 = fmaf(n1.w, inv.y, -ood.y);
          float c2 = fmaf(n2.z, inv.z, -ood.z), d2 = fmaf(n2.w, inv.z, -ood.z);
          float tn1 = fmaxf(fmaxf(fminf(c0, d0), fminf(c1, d1)), fmaxf(fminf(c2, d2), 0.0f));
          float tf1 = fminf(fminf(fmaxf(c0, d0), fmaxf(c1, d1)), fminf(fmaxf(c2, d2), tlimit));
          bool h0 = tn0 <= tf0 * 1.0000005f, h1 = tn1 <= tf1 * 1.0000005f;
          if (h0 && h1) {
            bool first0 = tn0 <= tn1;
            int near_ref = first0 ? n3.x : n3.y, far_ref = first0 ? n3.y : n3.x;
            int near_cnt = first0 ? n3.z : n3.w, far_cnt = first0 ? n3.w : n3.z;
            if (sp < kStack) {
              stack_ref[sp] = far_ref < 0 ? ~((~far_ref) << 3 | (far_cnt - 1)) : far_ref;
              stack_tn[sp] = first0 ? tn1 : tn0;
              sp++;
            }
            cur = near_ref;
            cnt = near_cnt;
          } else if (h0) {
            cur = n3.x;
            cnt = n3.z;
          } else if (h1) {
            cur = n3.y;
            cnt = n3.w;
          } else {
            cur = pop();
          }
        } else if (cur != DONE) {
          if (pl != DONE) break;  // a second leaf waits for the next round
          pl = cur;
          pcnt = cnt;
          cur = pop();
        }
        if (cur == DONE) break;
        if (pl != DONE) {
          if (!SPEC) break;
          if (!__any_sync(__activemask(), pl == DONE)) break;
        }
      }
      if (pl != DONE) {
        int first = ~pl;
        for (int k = 0; k < pcnt; k++) {
          const float4* tp = A.tris + 3 * (size_t)(first + k);
          float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
          float t;
          if (tri_exact_n(f3(v0), f3(v1), f3(v2), A.tri_nrm + first + k, o, d, t)) {
            uint32_t leaf = __float_as_uint(v1.w), pos = __float_as_uint(v2.w);
            if (!best.hit || t < best.t ||
                (t == best.t && (leaf > best.leaf || (leaf == best.leaf && pos < best.pos)))) {
              best = {__float_as_int(v0.w), t, leaf, pos, true};
              tlimit = t + A.prune_rel * (1.0f + t);
            }
          }
        }
      }
    }

    if (active && cur == DONE) {
      if (slot_rec) {  // one 16-byte record by binned slot; the check scatters it to ray order
        slot_rec[slot] = make_int4(best.hit ? best.tid : -1, __float_as_int(best.hit ? best.t : -1.0f),
                                   (int)(best.hit ? best.leaf : kNoLeaf), 0);
      } else {
        out_tid[ray] = best.hit ? best.tid : -1;
        out_dist[ray] = best.hit ? best.t : -1.0f;
        hit_leaf[ray] = best.hit ? best.leaf : kNoLeaf;
      }
      active = false;
    }
  }
  unsigned sum = n_exact;
  for (int s2 = 16; s2 > 0; s2 >>= 1) sum += __shfl_xor_sync(FULL, sum, s2);
  if (lane == 0 && sum) atomicAdd(&counters[1], (unsigned long long)sum);
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

// The reference's own walk (KDTree.cpp:295-333) on the reference tree: every node whose
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

// ---- ray binning (rx_bin.cuh): counting sort by (origin cell, direction bin) --------
__global__ void k_ray_keys(DevAccel A, const rx_ray* __restrict__ rays, uint32_t n, uint32_t* __restrict__ keys,
                           uint32_t* __restrict__ hist, int cbits, int dbits, int dir_map) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4* rp = reinterpret_cast<const float4*>(rays + i);
    uint32_t k = ray_key(A.lo, A.hi, __ldg(rp), __ldg(rp + 1), cbits, dbits, dir_map);
    keys[i] = k;
    atomicAdd(&hist[k], 1u);
  }
}

__global__ void k_ray_scatter(const uint32_t* __restrict__ keys, uint32_t n_host, const unsigned* count,
                              uint32_t* __restrict__ cursor, uint32_t* __restrict__ order) {
  const uint32_t n = count ? *count : n_host;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    order[atomicAdd(&cursor[keys[i]], 1u)] = i;
}

cudaError_t launch_trace_closest(const DevAccel& A, const rx_ray* rays, uint32_t n, int32_t* tid, float* dist,
                                 uint32_t* queue, unsigned long long* counters, const TraceConfig& cfg,
                                 cudaStream_t s, const cudaEvent_t* ev, bool bin) {
  if (n == 0) return cudaSuccess;
  cudaMemsetAsync(counters, 0, sizeof(unsigned long long), s);  // eager queue length
  uint32_t* hit_leaf = queue;  // scratch: n entries of winners' reference leaves
  uint32_t* eager = queue + n;  // then up to n queued rays
  if (cfg.variant != 0) cudaMemsetAsync(counters + 4, 0, sizeof(unsigned long long), s);  // batch cursor
  const uint32_t* order = nullptr;
  int4* slot_rec = nullptr;
  if (bin && cfg.variant != 0 && cfg.bin_min && n >= cfg.bin_min) {
    uint32_t* keys = queue + 2 * (size_t)n;
    uint32_t* perm = queue + 3 * (size_t)n;
    uint32_t* hist = queue + 8 * (size_t)n;
    const uint32_t bins = 1u << (3 * cfg.bin_cell_bits + (cfg.bin_dir_map ? 2 : 3) * cfg.bin_dir_bits);
    cudaMemsetAsync(hist, 0, bins * sizeof(uint32_t), s);  // at most kRayBinsMax
    k_ray_keys<<<cfg.sms * 8, 256, 0, s>>>(A, rays, n, keys, hist, cfg.bin_cell_bits, cfg.bin_dir_bits,
                                           cfg.bin_dir_map);
    scan_bins(hist, hist + kRayBinsMax, s, bins);
    k_ray_scatter<<<cfg.sms * 8, 256, 0, s>>>(keys, n, nullptr, hist, perm);
    order = perm;
    if (cfg.check_thread)  // the walk writes its answers by slot: 16-byte records after perm
      slot_rec = reinterpret_cast<int4*>(queue + 4 * (size_t)n);
  }
  if (ev) cudaEventRecord(ev[0], s);
  if (cfg.variant == 0) {
    k_trace_closest<<<(n + 127) / 128, 128, 0, s>>>(A, rays, n, tid, dist, hit_leaf, counters);
  } else {
    unsigned blocks = (unsigned)cfg.sms * (unsigned)cfg.blocks_per_sm;
    unsigned need = (n + 127) / 128;
    blocks = blocks < need ? blocks : need;
    // the walk's stack lives in local memory: the shallower one when the BVH allows
    const bool shallow = cfg.walk_stack != 64 && A.bvh_depth < 32;
    const bool walk4 = A.bvh4 && 3 * A.bvh4_depth + 1 <= 64;  // the 4-wide walk's stack bound
    const bool walk8 = A.bvh8 && 7 * A.bvh8_depth + 1 <= 80;  // the 8-wide walk's
    if ((cfg.variant == 5 && walk8) || (cfg.variant == 4 && !walk4 && walk8))
      k_trace_persistent8<16><<<blocks, 128, 0, s>>>(A, rays, n, order, tid, dist, hit_leaf, slot_rec, counters);
    else if ((cfg.variant == 4 || cfg.variant == 5) && walk4)
      k_trace_persistent4<16><<<blocks, 128, 0, s>>>(A, rays, n, order, tid, dist, hit_leaf, slot_rec, counters);
    else if (cfg.variant == 3 && walk4)
      k_trace_persistent4<0><<<blocks, 128, 0, s>>>(A, rays, n, order, tid, dist, hit_leaf, slot_rec, counters);
    else if (cfg.variant == 1 && shallow)
      k_trace_persistent<false, 32><<<blocks, 128, 0, s>>>(A, rays, n, order, tid, dist, hit_leaf, slot_rec, counters);
    else if (cfg.variant == 1)
      k_trace_persistent<false, kStack><<<blocks, 128, 0, s>>>(A, rays, n, order, tid, dist, hit_leaf, slot_rec, counters);
    else if (shallow)
      k_trace_persistent<true, 32><<<blocks, 128, 0, s>>>(A, rays, n, order, tid, dist, hit_leaf, slot_rec, counters);
    else
      k_trace_persistent<true, kStack><<<blocks, 128, 0, s>>>(A, rays, n, order, tid, dist, hit_leaf, slot_rec, counters);
  }
  if (ev) cudaEventRecord(ev[1], s);
  if (cfg.check_thread)
    k_check_visible_thread<<<cfg.sms * 16, 128, 0, s>>>(A, rays, n, order, hit_leaf, slot_rec, tid, dist, eager,
                                                        counters);
  else
    k_check_visible<<<cfg.sms * 16, 128, 0, s>>>(A, rays, n, hit_leaf, eager, counters);
  if (ev) cudaEventRecord(ev[2], s);
  k_trace_eager<<<cfg.sms, 128, 0, s>>>(A, rays, tid, dist, eager, counters);
  if (ev) cudaEventRecord(ev[3], s);
  return cudaGetLastError();
}

// The triangle test's unit normal per slot, by the test's own functions (so the bits
// are those the test would form: IEEE operations, never contracted).
__global__ void k_slot_normals(const float4* __restrict__ tris, uint32_t nslots, float4* __restrict__ nrm) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nslots; i += gridDim.x * blockDim.x) {
    const float4* tp = tris + 3 * (size_t)i;
    const F3 v0 = f3(tp[0]), v1 = f3(tp[1]), v2 = f3(tp[2]);
    const F3 n = xnormalize(xcross(xsub(v1, v0), xsub(v2, v1)));
    nrm[i] = make_float4(n.x, n.y, n.z, 0.0f);
  }
}

cudaError_t launch_slot_normals(const float4* tris, uint32_t nslots, float4* nrm, cudaStream_t s) {
  if (nslots == 0) return cudaSuccess;
  k_slot_normals<<<(nslots + 255) / 256 < 4096 ? (nslots + 255) / 256 : 4096, 256, 0, s>>>(tris, nslots, nrm);
  return cudaGetLastError();
}

cudaError_t launch_trace_reforder(const DevAccel& A, const rx_ray* rays, uint32_t n, int32_t* tid, float* dist,
                                  unsigned long long* counters, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_trace_reforder<<<(n + 127) / 128, 128, 0, s>>>(A, rays, n, tid, dist, counters);
  return cudaGetLastError();
}

}  // namespace rx
