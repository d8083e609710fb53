// Device-side scene and acceleration data shared by the kernels of the library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rx {

// Traversal stack entries; the BVH builder keeps the depth below this.
constexpr int kStackDepth = 64;

// Closest-hit structures, all in HBM, 16-byte aligned for 128-bit loads.
//  bvh  : 4 float4 per node: (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y),
//         (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y), (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z),
//         (child0, child1, count0, count1) as int bits; child < 0 is ~first leaf slot.
//  tris : 3 float4 per BVH leaf slot, vertices in the triangle's own order:
//         v0.w = global triangle id, v1.w = reference leaf index (DFS order),
//         v2.w = position in the reference's DFS triangle order (all int bits).
//  ref  : 2 float4 per reference-tree node: (min.xyz, parent id bits), (max.xyz, 0).
//  ref_leaf_node : reference leaf index -> reference node id.
struct DevAccel {
  const float4* bvh;
  const float4* tris;
  const float4* tri_nrm;  // per triangle slot: xnormalize(xcross(v1 - v0, v2 - v1)) (k_slot_normals)
  const float4* ref;
  const int32_t* ref_leaf_node;
  const uint32_t* ref_leaf_range;  // 2 per leaf: [begin, end) in reference DFS order
  const float4* ref_tris;          // 3 float4 per triangle in reference DFS order (v*.w unused but v0.w = id)
  const uint32_t* anc_range;       // 2 per leaf: [begin, end) into anc_nodes
  const int32_t* anc_nodes;        // per leaf, its root path (leaf first) as node ids
  const float4* anc_box;           // the same entries as 2 float4 each: that node's ref box
  uint32_t num_nodes, num_tris, num_ref_nodes, num_ref_leaves;
  float prune_rel;                 // pruning margin: t_limit = best + prune_rel*(1+best)
  float lo[3], hi[3];              // scene bounds (ray binning)
  uint32_t bvh_depth;              // deepest BVH level (the walk's stack must exceed it)
  const float4* bvh4;              // 4-wide BVH, 8 float4 per node (rx_accel.h), or null
  uint32_t bvh4_depth;
  const float4* bvh8;              // 8-wide BVH, 16 float4 per node (rx_accel.h), or null
  uint32_t bvh8_depth;
};

}  // namespace rx
