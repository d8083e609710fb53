// ORACLE — test infrastructure only. The restated reference triangle tree (reference
// include/KDTree.h, src/KDTree.cpp) shared by the oracle's translation units: vector
// helpers with the reference's operation order, the tree, the box and triangle tests
// and the traversal. See rxo_kdtree.cpp for the build and the C entry points.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

namespace rxo {

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
  uint32_t tri_begin = 0, tri_end = 0;  // range in tri_order (leaves only)
};

}  // namespace rxo

struct rxo_tree {
  std::vector<rxo::V3> verts;
  std::vector<uint32_t> tris;  // 3 per triangle
  std::vector<rxo::Node> nodes;     // DFS pre-order, left child first (KDTree.cpp:346-377)
  std::vector<uint32_t> tri_order;  // leaf triangle ids, leaves in DFS order
  int max_depth = 0;
};

namespace rxo {

// KDTree::Node::BoundingBox::intersect, KDTree.cpp:34-52. Faces in the order of the
// box's float layout (min.xyz then max.xyz); no epsilon.
inline float box_test(const Node& n, V3 o, V3 d) {
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
inline float tri_test(const rxo_tree* T, uint32_t t, V3 o, V3 d) {
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
// equal distances keep the right child; in a leaf the first strictly closer wins. A
// triangle counts only where legal(t, dist) holds (the condition of KDTree.cpp:290,
// evaluated after the distance).
template <class Legal>
float node_isect(const rxo_tree* T, int ni, V3 o, V3 d, unsigned& tid, const Legal& legal) {
  const Node& n = T->nodes[ni];
  if (box_test(n, o, d) < 0) return -1;
  if (n.left < 0) {
    float minDist = -1;
    for (uint32_t k = n.tri_begin; k < n.tri_end; k++) {
      uint32_t t = T->tri_order[k];
      float dist = tri_test(T, t, o, d);
      if (dist >= 0 && !legal(t, dist)) dist = -1;
      if (dist >= 0 && (dist < minDist || minDist < 0)) { minDist = dist; tid = t; }
    }
    return minDist;
  }
  unsigned lt = 0, rt = 0;
  float ld = node_isect(T, n.left, o, d, lt, legal);
  float rd = node_isect(T, n.right, o, d, rt, legal);
  if (ld >= 0 && rd >= 0) { tid = ld < rd ? lt : rt; return ld < rd ? ld : rd; }
  else if (rd < 0) { tid = lt; return ld; }
  else if (ld < 0) { tid = rt; return rd; }
  return -1;
}

struct AlwaysLegal {
  bool operator()(uint32_t, float) const { return true; }
};

}  // namespace rxo
