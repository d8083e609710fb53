// Host-side acceleration structures for the closest-hit path.
//
// Two trees are built over the same triangles:
//  * RefOrder: the reference's own triangle tree (reference src/KDTree.cpp:129-246,
//    splitBest + build), rebuilt exactly. It is never traversed on the GPU; it
//    supplies (a) the rank that breaks equal-distance ties the way the reference's
//    recursive traversal does (KDTree.cpp:295-333: right child wins ties, first
//    triangle in a leaf wins) and (b) the node boxes whose reference box test
//    (KDTree.cpp:34-52, no epsilon) decides whether the reference can see a
//    triangle at all.
//  * Bvh: a binned-SAH bounding volume hierarchy with padded boxes, the structure the
//    GPU actually walks.
#pragma once
#include <cstdint>
#include <vector>

namespace rx {

struct RefNodeHost {
  float mn[3], mx[3];
  int32_t parent;   // -1 at the root
  int32_t left, right;  // -1 for leaves
  uint32_t tri_begin, tri_end;  // leaves: range in RefOrder::tri_order
};

struct RefOrder {
  std::vector<RefNodeHost> nodes;   // DFS pre-order, left first
  std::vector<uint32_t> tri_order;  // triangle ids, leaves in DFS order
  std::vector<uint32_t> leaf_node;  // leaf index (DFS order of leaves) -> node id
  std::vector<uint32_t> tri_leaf;   // triangle id -> leaf index
  std::vector<uint32_t> tri_pos;    // triangle id -> position in tri_order
  int max_depth = 0;
};

// policy 0: the reference as compiled by GCC/libstdc++ (KDTree.cpp:191 `abs` binds to
// int abs, the x axis is always kept); policy 1: best-ratio axis (libc++/MSVC builds).
bool build_ref_order(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt, int policy,
                     int threads, RefOrder& out);

// Aila-Laine style binary node: both children's boxes live in the parent.
struct BvhNodeHost {
  float c0lo[3], c0hi[3], c1lo[3], c1hi[3];
  int32_t child[2];   // >= 0: inner node id; < 0: ~leaf_first (triangle slot)
  int32_t count[2];   // triangles in a leaf child, 0 for inner children
};

struct Bvh {
  std::vector<BvhNodeHost> nodes;
  std::vector<uint32_t> tri_order;  // triangle id per slot
  int max_depth = 0;
  int leaf_size = 4;
};

bool build_bvh(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt, int leaf_size, int threads,
               Bvh& out);

// 4-wide BVH collapsed from the binary one: each node holds up to four children (inner
// nodes or leaves of the binary tree), found by repeatedly opening the child with the
// largest surface area. Node layout on the device: 8 float4 = 128 B (lo.x, hi.x, lo.y,
// hi.y, lo.z, hi.z of the four children, then the four child refs, then four spare
// words, zero; an empty child slot has the inverted box lo = +inf, hi = -inf, which every
// slab test rejects, and ref kBvh4Empty). A child ref is an inner node's index (>= 0), a leaf packed with its
// triangle count as ~(first_slot << 3 | (count - 1)) (negative; counts 1..8, slots below
// 2^28: the walks' stack entries use the same packing, so refs are pushed as they are),
// or kBvh4Empty for an empty slot.
constexpr int32_t kBvh4Empty = 0x7fffffff;
#ifdef __CUDACC__
#define RX_HD __host__ __device__
#else
#define RX_HD
#endif
RX_HD inline int32_t pack_leaf(int32_t first_slot, int32_t count) { return ~((first_slot << 3) | (count - 1)); }
RX_HD inline int32_t leaf_first(int32_t packed) { return (~packed) >> 3; }
RX_HD inline int32_t leaf_count(int32_t packed) { return ((~packed) & 7) + 1; }
struct Bvh4 {
  std::vector<float> data;  // 32 floats per node
  int max_depth = 0;
  size_t num_nodes() const { return data.size() / 32; }
};
void collapse_bvh4(const Bvh& b2, Bvh4& out);
// The same with up to eight children per node: 16 float4 = 256 B per node (lo.x, hi.x,
// lo.y, hi.y, lo.z, hi.z of the eight children, then eight packed refs, eight spare).
void collapse_bvh8(const Bvh& b2, Bvh4& out);

}  // namespace rx
