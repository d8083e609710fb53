// ORACLE — test infrastructure only. A CPU restatement of the reference's triangle
// KDTree (reference include/KDTree.h, src/KDTree.cpp) used to check the GPU closest-hit
// path. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
// it; the product never does.
//
// Parity pins: the restatement is checked against the reference's own KDTree compiled
// from its sources (oracle/ref/hit_driver.cpp) through the committed golden fixtures in
// tests/golden/ (hit ids, distances and the reference's serialized tree).
//
// Build: see oracle/Makefile (-O2 -ffp-contract=off, no fast-math: every float
// operation below is one IEEE-754 single-precision operation, as in the reference's
// x86-64 build).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "rxo_tree.h"

using namespace rxo;

namespace {

// KDTree::splitBest, KDTree.cpp:129-228. Split policy:
//  0 = the reference as compiled with GCC/libstdc++: `abs(ratio-0.5)` at
//      KDTree.cpp:191 binds to int abs(int), truncates both sides to 0 and 9, so the
//      first axis (x) is always kept;
//  1 = the intended behaviour (libc++/MSVC bind abs(double)): the axis whose
//      left-count ratio is closest to 0.5, first axis on ties.
struct Builder {
  rxo_tree* T;
  int policy;
  std::vector<uint32_t> stamp;
  uint32_t cur = 0;
  std::vector<uint32_t> tmp;
  std::vector<float> coords;

  void bounds(const std::vector<uint32_t>& idx, Node& n) {
    // KDTree.cpp:139-153: start from the first triangle's first vertex
    V3 p0 = T->verts[T->tris[3 * idx[0]]];
    float mn[3] = {p0.x, p0.y, p0.z}, mx[3] = {p0.x, p0.y, p0.z};
    for (uint32_t t : idx)
      for (int k = 0; k < 3; k++) {
        V3 p = T->verts[T->tris[3 * t + k]];
        for (int a = 0; a < 3; a++) {
          mn[a] = p[a] < mn[a] ? p[a] : mn[a];  // boundvec<1>(p, min), KDTree.cpp:4-20
          mx[a] = p[a] > mx[a] ? p[a] : mx[a];
        }
      }
    for (int a = 0; a < 3; a++) { n.mn[a] = mn[a]; n.mx[a] = mx[a]; }
  }

  // returns node id
  int build(std::vector<uint32_t>& idx, int depth) {
    int id = (int)T->nodes.size();
    T->nodes.push_back(Node());
    if (depth > T->max_depth) T->max_depth = depth;
    Node n;
    bounds(idx, n);
    bool leaf = idx.size() <= 1;  // maxLeafTriangleNum = 1, KDTree.cpp:22-27
    int best_dim = 0;
    float best_ratio = 10, best_split = 0;
    if (!leaf) {
      int ndims = policy == 0 ? 1 : 3;  // policy 0 never keeps axes 1, 2
      for (int dim = 0; dim < ndims; dim++) {
        // unique vertex indices of the node (unordered_set at KDTree.cpp:142-152)
        cur++;
        coords.clear();
        for (uint32_t t : idx)
          for (int k = 0; k < 3; k++) {
            uint32_t v = T->tris[3 * t + k];
            if (stamp[v] != cur) { stamp[v] = cur; coords.push_back(T->verts[v][dim]); }
          }
        size_t mid = coords.size() >> 1;
        std::nth_element(coords.begin(), coords.begin() + mid, coords.end());
        float split = coords[mid];  // KDTree.cpp:167-171
        unsigned left = 0;
        for (uint32_t t : idx) {
          unsigned mask = 0;
          for (int k = 0; k < 3; k++) mask += (T->verts[T->tris[3 * t + k]][dim] <= split) << k;
          if (mask != 0) left++;
        }
        float ratio = left / float(idx.size());
        bool better;
        if (policy == 0) better = (dim == 0);  // int abs: 0 < 9 for axis 0 only
        else better = std::fabs(ratio - 0.5) < std::fabs(best_ratio - 0.5);
        if (better) { best_ratio = ratio; best_dim = dim; best_split = split; }
      }
      if (best_ratio == 0 || best_ratio == 1) leaf = true;  // KDTree.cpp:199-203
    }
    if (leaf) {
      n.tri_begin = (uint32_t)T->tri_order.size();
      for (uint32_t t : idx) T->tri_order.push_back(t);
      n.tri_end = (uint32_t)T->tri_order.size();
      T->nodes[id] = n;
      return id;
    }
    // KDTree.cpp:208-224: right gets triangles with no vertex <= split, in order
    std::vector<uint32_t> L, R;
    L.reserve(idx.size());
    for (uint32_t t : idx) {
      unsigned mask = 0;
      for (int k = 0; k < 3; k++) mask += (T->verts[T->tris[3 * t + k]][best_dim] <= best_split) << k;
      (mask == 0 ? R : L).push_back(t);
    }
    std::vector<uint32_t>().swap(idx);
    T->nodes[id] = n;
    int l = build(L, depth + 1);
    int r = build(R, depth + 1);
    T->nodes[id].left = l;
    T->nodes[id].right = r;
    return id;
  }
};

}  // namespace

extern "C" {

// Build the reference tree over (verts, tris). Returns NULL on empty input.
rxo_tree* rxo_tree_build(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt, int policy) {
  if (nt == 0 || nv == 0) return nullptr;
  rxo_tree* T = new rxo_tree();
  T->verts.resize(nv);
  for (uint32_t i = 0; i < nv; i++) T->verts[i] = {verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]};
  T->tris.assign(tris, tris + 3 * (size_t)nt);
  Builder b{T, policy};
  b.stamp.assign(nv, 0);
  std::vector<uint32_t> idx(nt);
  for (uint32_t i = 0; i < nt; i++) idx[i] = i;
  T->nodes.reserve(2 * (size_t)nt);
  T->tri_order.reserve(nt);
  b.build(idx, 0);
  return T;
}

void rxo_tree_free(rxo_tree* T) { delete T; }
uint32_t rxo_tree_num_nodes(const rxo_tree* T) { return (uint32_t)T->nodes.size(); }
uint32_t rxo_tree_num_leaf_tris(const rxo_tree* T) { return (uint32_t)T->tri_order.size(); }
int rxo_tree_max_depth(const rxo_tree* T) { return T->max_depth; }

// Same content as KDTree::serializeForGPU (KDTree.cpp:346-382): per node 12 floats
// (parent, rightChild, leafStart, leafEnd, min.xyz, 0, max.xyz, 0) and, per leaf
// triangle, its id, in DFS order.
void rxo_tree_serialize(const rxo_tree* T, float* nodes12, float* leaf_tid) {
  std::vector<int> parent(T->nodes.size(), -1);
  for (size_t i = 0; i < T->nodes.size(); i++)
    if (T->nodes[i].left >= 0) { parent[T->nodes[i].left] = (int)i; parent[T->nodes[i].right] = (int)i; }
  for (size_t i = 0; i < T->nodes.size(); i++) {
    const Node& n = T->nodes[i];
    float* o = nodes12 + 12 * i;
    o[0] = (float)parent[i];
    if (n.left >= 0) { o[1] = (float)n.right; o[2] = -1; o[3] = -1; }
    else { o[1] = -1; o[2] = (float)n.tri_begin; o[3] = (float)n.tri_end; }
    o[4] = n.mn[0]; o[5] = n.mn[1]; o[6] = n.mn[2]; o[7] = 0;
    o[8] = n.mx[0]; o[9] = n.mx[1]; o[10] = n.mx[2]; o[11] = 0;
  }
  for (size_t k = 0; k < T->tri_order.size(); k++) leaf_tid[k] = (float)T->tri_order[k];
}

// Closest hit for n rays (rays6: origin xyz, direction xyz), the public
// KDTree::intersect(ray, tid, NULL) of KDTree.cpp:335-339. tid = -1 on a miss.
void rxo_trace(const rxo_tree* T, const float* rays6, uint32_t n, int32_t* tid, float* dist, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (long i = 0; i < (long)n; i++) {
    V3 o = {rays6[6 * i], rays6[6 * i + 1], rays6[6 * i + 2]};
    V3 d = {rays6[6 * i + 3], rays6[6 * i + 4], rays6[6 * i + 5]};
    unsigned t = 0;
    float r = node_isect(T, 0, o, d, t, AlwaysLegal{});
    dist[i] = r;
    tid[i] = r >= 0 ? (int32_t)t : -1;
  }
}

// Closest hit over every triangle that passes the triangle test, ignoring the tree's
// box tests: candidates ordered by (distance, later leaf first, earlier leaf slot
// first), the order in which the reference's traversal (KDTree.cpp:295-333) would
// pick them if every box passed. Where this differs from rxo_trace, the reference's
// box tests hide the closest triangle from the ray.
void rxo_trace_unboxed(const rxo_tree* T, const float* rays6, uint32_t n, int32_t* tid, float* dist, int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (long i = 0; i < (long)n; i++) {
    V3 o = {rays6[6 * i], rays6[6 * i + 1], rays6[6 * i + 2]};
    V3 d = {rays6[6 * i + 3], rays6[6 * i + 4], rays6[6 * i + 5]};
    float best = -1;
    int32_t bt = -1;
    for (size_t ni = 0; ni < T->nodes.size(); ni++) {  // DFS pre-order: leaves in DFS order
      const Node& nd = T->nodes[ni];
      if (nd.left >= 0) continue;
      float lbest = -1;
      int32_t lt = -1;
      for (uint32_t k = nd.tri_begin; k < nd.tri_end; k++) {
        uint32_t tt = T->tri_order[k];
        float r = tri_test(T, tt, o, d);
        if (r >= 0 && (r < lbest || lbest < 0)) { lbest = r; lt = (int32_t)tt; }
      }
      if (lbest >= 0 && (best < 0 || lbest <= best)) { best = lbest; bt = lt; }  // ties: later leaf
    }
    dist[i] = best;
    tid[i] = bt;
  }
}

// Reference box test and triangle test exposed for unit tests.
float rxo_box_test(const float* mn3, const float* mx3, const float* o3, const float* d3) {
  Node n;
  for (int a = 0; a < 3; a++) { n.mn[a] = mn3[a]; n.mx[a] = mx3[a]; }
  return box_test(n, {o3[0], o3[1], o3[2]}, {d3[0], d3[1], d3[2]});
}

int rxo_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
