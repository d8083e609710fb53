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

namespace {

struct V3 {
  float x, y, z;
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

// nvVector.h:491-499 (cross), :502-508 (dot accumulates from 0), :511-527 (normalize
// divides each component by sqrt of the accumulated square norm).
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 cross(V3 l, V3 r) { return {l.y * r.z - l.z * r.y, l.z * r.x - l.x * r.z, l.x * r.y - l.y * r.x}; }
inline float dot(V3 a, V3 b) {
  float r = 0;
  r += a.x * b.x;
  r += a.y * b.y;
  r += a.z * b.z;
  return r;
}
inline V3 normalized(V3 v) {
  float sq = 0;
  sq += v.x * v.x;
  sq += v.y * v.y;
  sq += v.z * v.z;
  float r = (float)std::sqrt((double)sq);  // correctly rounded float sqrt
  if (r > 0) { v.x /= r; v.y /= r; v.z /= r; }
  return v;
}

struct Node {
  float mn[3], mx[3];
  int left = -1, right = -1;          // child node ids, -1 for a leaf
  uint32_t tri_begin = 0, tri_end = 0;  // range in Tree::tri_order (leaves only)
};

}  // namespace

struct rxo_tree {
  std::vector<V3> verts;
  std::vector<uint32_t> tris;  // 3 per triangle
  std::vector<Node> nodes;     // DFS pre-order, left child first (KDTree.cpp:346-377)
  std::vector<uint32_t> tri_order;  // leaf triangle ids, leaves in DFS order
  int max_depth = 0;
};

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

// KDTree::Node::BoundingBox::intersect, KDTree.cpp:34-52. Faces in the order of the
// box's float layout (min.xyz then max.xyz); no epsilon.
float box_test(const Node& n, V3 o, V3 d) {
  const float b[6] = {n.mn[0], n.mn[1], n.mn[2], n.mx[0], n.mx[1], n.mx[2]};
  float minDist = -1;
  for (unsigned i = 0; i < 6; i++) {
    int a = i % 3;
    if (d[a] == 0) continue;
    float dist = (b[i] - o[a]) / d[a];
    V3 ip = {o.x + dist * d.x, o.y + dist * d.y, o.z + dist * d.z};
    int a1 = (i + 1) % 3, a2 = (i + 2) % 3;
    bool inter = dist >= 0;
    inter &= n.mn[a1] <= ip[a1];
    inter &= n.mx[a1] >= ip[a1];
    inter &= n.mn[a2] <= ip[a2];
    inter &= n.mx[a2] >= ip[a2];
    minDist = (inter && (dist < minDist || minDist < 0)) ? dist : minDist;
  }
  return minDist;
}

// KDTree::intersect(ray, triangle), KDTree.cpp:267-293 (no condition).
float tri_test(const rxo_tree* T, uint32_t t, V3 o, V3 d) {
  V3 vs[3];
  for (int i = 0; i < 3; i++) vs[i] = T->verts[T->tris[3 * t + i]];
  unsigned mask_pos = 0, mask_neg = 0;
  V3 lines[3], r2v = {0, 0, 0}, n;
  for (unsigned i = 0; i < 3; i++) {
    lines[i] = sub(vs[(i + 1) % 3], vs[i]);
    r2v = sub(vs[i], o);
    n = cross(lines[i], r2v);
    float s = dot(d, n);
    mask_pos += (s >= 0) << i;
    mask_neg += (s <= 0) << i;
  }
  n = normalized(cross(lines[0], lines[1]));
  float orthoDist = dot(n, r2v);
  float dd = dot(n, d);
  if (dd == 0 || orthoDist / dd < 0 || (mask_pos != 7 && mask_neg != 7)) return -1;
  return orthoDist / dd;
}

// KDTree::intersect(ray, node), KDTree.cpp:295-333: both children always visited;
// equal distances keep the right child; in a leaf the first strictly closer wins.
float node_isect(const rxo_tree* T, int ni, V3 o, V3 d, unsigned& tid) {
  const Node& n = T->nodes[ni];
  if (box_test(n, o, d) < 0) return -1;
  if (n.left < 0) {
    float minDist = -1;
    for (uint32_t k = n.tri_begin; k < n.tri_end; k++) {
      uint32_t t = T->tri_order[k];
      float dist = tri_test(T, t, o, d);
      if (dist >= 0 && (dist < minDist || minDist < 0)) { minDist = dist; tid = t; }
    }
    return minDist;
  }
  unsigned lt = 0, rt = 0;
  float ld = node_isect(T, n.left, o, d, lt);
  float rd = node_isect(T, n.right, o, d, rt);
  if (ld >= 0 && rd >= 0) { tid = ld < rd ? lt : rt; return ld < rd ? ld : rd; }
  else if (rd < 0) { tid = lt; return ld; }
  else if (ld < 0) { tid = rt; return rd; }
  return -1;
}

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
#pragma omp parallel for schedule(dynamic, 16)
#endif
  for (long i = 0; i < (long)n; i++) {
    V3 o = {rays6[6 * i], rays6[6 * i + 1], rays6[6 * i + 2]};
    V3 d = {rays6[6 * i + 3], rays6[6 * i + 4], rays6[6 * i + 5]};
    unsigned t = 0;
    float r = node_isect(T, 0, o, d, t);
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
#pragma omp parallel for schedule(dynamic, 16)
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
