// The persistent walk over a W-wide BVH (W = 4: 128-byte nodes, one cache line; W = 8:
// 256-byte nodes, half the levels), shared by the closest-hit batch (rx_trace.cu), the
// path tracer's extension rays (rx_pt.cu) and the connections' shadow rays (rx_vcm.cu,
// any hit). Warps stay resident and refill lanes whose
// ray has finished from a cursor (one atomic per warp and refill), so a warp never idles
// behind its longest ray. One node visit tests W child boxes, visits the nearest hit
// child next and stacks the others far to near with their entry distances. Child refs
// come packed from the node (a leaf's first triangle and count in one word, rx_accel.h)
// and go on the stack as they are; a leaf is unpacked when its triangles are tested.
// Each axis's near plane is picked once per ray by the sign of its inverse direction and
// loaded as such, so the slab values need no ordering; an empty child slot holds an
// inverted box that the slab test rejects by itself. An any-hit policy ends its ray by
// returning a limit below every entry distance.
//
// Traversal steps are warp-uniform: a lane without a leaf to test walks until it finds
// one; meanwhile a lane that already holds one keeps walking inner nodes (its leaf
// postponed, as in Aila and Laine's speculative traversal), so fewer lanes idle. A lane
// stops when it reaches a second leaf. Pruning uses the limit before the postponed
// leaf, which only visits more candidates, never fewer; leaves are tested in the order
// they are reached, as a walk without postponing tests them.
//
// kShort > 0: the first kShort entries of each thread's stack sit in shared memory (one
// column per thread of a 128-thread block, conflict-free), deeper ones in local memory.
// kStack bounds the stack: (W - 1) entries per level below the root.
//
// The lane policy L supplies the ray source and the leaf test:
//   bool begin(uint32_t r, F3& o, F3& d)   take ray r of the batch (false: r is past it)
//   const float4* nodes() const            the lane's BVH (layout of rx_accel.h)
//   float limit() const                    entry distances beyond it are pruned
//   void leaf(int first, int count, F3 o, F3 d)  test the leaf's triangles
//   void end()                             the lane's ray is done: write its answer
#pragma once
#include <climits>
#include <cuda_runtime.h>
#include <stdint.h>

#include "rx_accel.h"
#include "rx_exact.cuh"

namespace rx {

template <int W, int kShort, int kStack, class Lane>
__device__ __forceinline__ void walk_persistent(Lane& L, unsigned long long* cursor) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int DONE = INT_MIN;
  constexpr int kShortN = kShort > 0 ? kShort : 1;
  __shared__ int s_ref[kShortN][128];
  __shared__ float s_tn[kShortN][128];
  const int lane = threadIdx.x & 31, tx = threadIdx.x;
  bool active = false, exhausted = false;
  F3 o{}, d{}, inv{}, ood{};
  int near_bits = 0;  // bit k: the near plane of axis k is the upper bound
  int stack_ref[kStack - kShort];
  float stack_tn[kStack - kShort];
  int sp = 0, cur = DONE;  // cur: an inner node, a packed leaf, or DONE

  auto pop = [&]() {
    const float lim = L.limit();
    while (sp > 0) {
      sp--;
      const bool sh = kShort > 0 && sp < kShort;
      if ((sh ? s_tn[sp][tx] : stack_tn[sp - kShort]) <= lim) return sh ? s_ref[sp][tx] : stack_ref[sp - kShort];
    }
    return DONE;
  };

  while (true) {
    const unsigned want = __ballot_sync(FULL, !active && !exhausted);
    if (want) {
      const int leader = __ffs(want) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(cursor, (unsigned long long)__popc(want));
      base = __shfl_sync(FULL, base, leader);
      if (!active && !exhausted) {
        const unsigned long long r = base + __popc(want & ((1u << lane) - 1));
        if (r < 0xffffffffull && L.begin((uint32_t)r, o, d)) {
          inv = safe_inv(d);
          ood = {o.x * inv.x, o.y * inv.y, o.z * inv.z};
          // the near plane of each axis: the lower bound where the inverse direction is
          // positive (safe_inv never returns zero), else the upper one
          near_bits = (inv.x < 0.0f ? 1 : 0) | (inv.y < 0.0f ? 2 : 0) | (inv.z < 0.0f ? 4 : 0);
          sp = 0;
          cur = 0;
          active = true;
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(FULL, active)) break;

    int pl = DONE;  // the next leaf to test (packed)
    while (true) {
      const bool need = active && pl == DONE && cur != DONE;
      if (!__any_sync(FULL, need)) break;
      if (!(need || (active && cur >= 0))) continue;
      if (cur < 0) {  // a leaf (only lanes that need one get here)
        pl = cur;
        cur = pop();
        continue;
      }
      const float4* np = L.nodes() + 2 * W * (size_t)cur;
      float nr[3][W], fr[3][W];  // each child's near and far plane per axis
      int r[W];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const int nb = (near_bits >> k) & 1, on = (W / 4) * nb, of = (W / 4) * (1 - nb);
#pragma unroll
        for (int q = 0; q < W / 4; q++) {
          float4 l = __ldg(np + 2 * (W / 4) * k + on + q), h = __ldg(np + 2 * (W / 4) * k + of + q);
          nr[k][4 * q] = l.x, nr[k][4 * q + 1] = l.y, nr[k][4 * q + 2] = l.z, nr[k][4 * q + 3] = l.w;
          fr[k][4 * q] = h.x, fr[k][4 * q + 1] = h.y, fr[k][4 * q + 2] = h.z, fr[k][4 * q + 3] = h.w;
        }
      }
#pragma unroll
      for (int q = 0; q < W / 4; q++) {
        int4 cr = __ldg(reinterpret_cast<const int4*>(np + 6 * (W / 4) + q));
        r[4 * q] = cr.x, r[4 * q + 1] = cr.y, r[4 * q + 2] = cr.z, r[4 * q + 3] = cr.w;
      }
      const float lim = L.limit();
      float tn[W];
      int nh = 0;
#pragma unroll
      for (int j = 0; j < W; j++) {
        // fma(x, inv, -ood) is monotonic in x, so the near plane gives the smaller value
        // of each slab: the same entry and exit distances as ordering both with min/max
        float a0 = fmaf(nr[0][j], inv.x, -ood.x), b0 = fmaf(fr[0][j], inv.x, -ood.x);
        float a1 = fmaf(nr[1][j], inv.y, -ood.y), b1 = fmaf(fr[1][j], inv.y, -ood.y);
        float a2 = fmaf(nr[2][j], inv.z, -ood.z), b2 = fmaf(fr[2][j], inv.z, -ood.z);
        float t0 = fmaxf(max3f(a0, a1, a2), 0.0f);
        float t1 = fminf(min3f(b0, b1, b2), lim);
        bool h = t0 <= t1 * 1.0000005f;  // an empty slot's inverted box gives t0 = +inf, t1 = -inf
        tn[j] = h ? t0 : INFINITY;
        nh += h ? 1 : 0;
      }
      // sorting network on registers (ties keep child order): near to far
      auto cs = [&](int a, int b) {
        if (tn[b] < tn[a]) {
          float t = tn[a];
          tn[a] = tn[b];
          tn[b] = t;
          int q = r[a];
          r[a] = r[b];
          r[b] = q;
        }
      };
      if constexpr (W == 4) {
        cs(0, 1), cs(2, 3), cs(0, 2), cs(1, 3), cs(1, 2);
      } else {  // Batcher's odd-even merge sort of eight (19 exchanges)
        cs(0, 1), cs(2, 3), cs(4, 5), cs(6, 7);
        cs(0, 2), cs(1, 3), cs(4, 6), cs(5, 7);
        cs(1, 2), cs(5, 6);
        cs(0, 4), cs(1, 5), cs(2, 6), cs(3, 7);
        cs(2, 4), cs(3, 5);
        cs(1, 2), cs(3, 4), cs(5, 6);
      }
      if (nh == 0) {
        cur = pop();
      } else {
#pragma unroll
        for (int k = W - 1; k >= 1; k--) {  // farthest first, so the nearer pop earlier
          if (k < nh && sp < kStack) {
            if (kShort > 0 && sp < kShort) {
              s_ref[sp][tx] = r[k];
              s_tn[sp][tx] = tn[k];
            } else {
              stack_ref[sp - kShort] = r[k];
              stack_tn[sp - kShort] = tn[k];
            }
            sp++;
          }
        }
        cur = r[0];
      }
    }
    // (the next node was popped under the limit before this leaf's test: a looser limit
    // only visits more candidates, never fewer)
    if (active && pl != DONE) L.leaf(leaf_first(pl), leaf_count(pl), o, d);
    if (active && cur == DONE) {
      L.end();
      active = false;
    }
  }
}

}  // namespace rx
