// Closest-hit traversal with the reference's answer, bit for bit.
//
// The reference (KDTree::intersect, reference src/KDTree.cpp:295-339) returns, over
// the triangles it can see, the smallest distance; among equal distances the one in
// the latest leaf of its DFS order (the right child wins ties) and, within a leaf, the
// first. A triangle is visible when it passes the ray/triangle test and every node
// box on its root path passes the reference box test.
//
// The GPU walks a padded binned-SAH BVH instead, closest child first, pruning
// children whose entry distance exceeds the best distance plus a small margin (so
// equal-distance candidates are never pruned), and orders candidates by
// (distance, -reference leaf, reference position). The winner's reference root path
// is then checked with the reference box test (cheap filter, exact test only when
// undecided). In the rare case it fails, the ray is re-walked checking visibility at
// every improvement ("eager"), which yields the reference's answer exactly.
#pragma once
#include "rx_device.h"
#include "rx_exact.cuh"

namespace rx {

constexpr int kStack = kStackDepth;


// Reference visibility of a triangle in reference leaf `leaf`: every box on the root
// path passes KDTree.cpp:34-52. The root path comes from the per-leaf ancestor list,
// read four boxes at a time so the loads are independent.
__device__ __forceinline__ bool ref_visible(const DevAccel& A, uint32_t leaf, F3 o, F3 d, F3 inv, bool zero_dir,
                                            unsigned* n_exact) {
  uint32_t b = __ldg(&A.anc_range[2 * leaf]), e = __ldg(&A.anc_range[2 * leaf + 1]);
  const ClearMargins mg = clear_margins(o, d);
  for (uint32_t k = b; k < e; k += 4) {
    float4 lo[4], hi[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const uint32_t q = k + j < e ? k + j : k;
      lo[j] = __ldg(&A.anc_box[2 * (size_t)q]);
      hi[j] = __ldg(&A.anc_box[2 * (size_t)q + 1]);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      if (k + j >= e) continue;
      if (zero_dir || !box_clear_pass(f3(lo[j]), f3(hi[j]), o, d, inv, mg)) {
        (*n_exact)++;
        if (!box_exact(f3(lo[j]), f3(hi[j]), o, d)) return false;
      }
    }
  }
  return true;
}

struct HitResult {
  int32_t tid;
  float t;
  uint32_t leaf, pos;
  bool hit;
};

// One traversal. EAGER: check reference visibility before accepting each improvement.
template <bool EAGER>
__device__ __forceinline__ HitResult trace_ref_exact(const DevAccel& A, F3 o, F3 d, unsigned* n_exact) {
  F3 inv = safe_inv(d);
  bool zero_dir = (d.x == 0.0f) | (d.y == 0.0f) | (d.z == 0.0f);
  F3 ood = {o.x * inv.x, o.y * inv.y, o.z * inv.z};
  HitResult best{-1, -1.0f, 0u, 0u, false};
  float tlimit = INFINITY;
  int stack_ref[kStack];
  float stack_tn[kStack];
  int sp = 0;
  int cur = 0, cnt = 0;  // root inner node
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
          stack_ref[sp] = far_ref;
          stack_tn[sp] = first0 ? tn1 : tn0;
          // leaf counts ride in the low bits of the stacked reference for leaves
          if (far_ref < 0) stack_ref[sp] = ~((~far_ref) << 3 | (far_cnt - 1));
          sp++;
        }
        cur = near_ref;
        cnt = near_cnt;
        continue;
      } else if (h0) {
        cur = n3.x;
        cnt = n3.z;
        continue;
      } else if (h1) {
        cur = n3.y;
        cnt = n3.w;
        continue;
      }
    } else {
      int first = ~cur;
      for (int k = 0; k < cnt; k++) {
        const float4* tp = A.tris + 3 * (size_t)(first + k);
        float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
        float t;
        if (tri_exact_n(f3(v0), f3(v1), f3(v2), A.tri_nrm + first + k, o, d, t)) {
          uint32_t leaf = __float_as_uint(v1.w), pos = __float_as_uint(v2.w);
          bool better = !best.hit || t < best.t || (t == best.t && (leaf > best.leaf || (leaf == best.leaf && pos < best.pos)));
          if (EAGER && better) better = ref_visible(A, leaf, o, d, inv, zero_dir, n_exact);
          if (better) {
            best = {__float_as_int(v0.w), t, leaf, pos, true};
            tlimit = t + A.prune_rel * (1.0f + t);
          }
        }
      }
    }
    // pop the next child that can still hold the answer
    bool found = false;
    while (sp > 0) {
      sp--;
      if (stack_tn[sp] <= tlimit) {
        int r = stack_ref[sp];
        if (r < 0) {
          int packed = ~r;
          cur = ~(packed >> 3);
          cnt = (packed & 7) + 1;
        } else {
          cur = r;
        }
        found = true;
        break;
      }
    }
    if (!found) break;
  }
  return best;
}

}  // namespace rx
