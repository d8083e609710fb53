// Host builders for the closest-hit path: the reference-order tree (exact rebuild of
// reference src/KDTree.cpp:129-246) and the binned-SAH BVH the GPU walks.
#include "rx_accel.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>

namespace rx {

// ----------------------------------------------------------------------------------
// Reference-order tree
// ----------------------------------------------------------------------------------
namespace {

struct RefCtx {
  const float* v;
  const uint32_t* t;
  int policy;
};

struct RefTmpNode {
  float mn[3], mx[3];
  int left = -1, right = -1;
  std::vector<uint32_t> leaf_tris;  // leaves only
  int depth = 0;
};

// One subtree, built by one thread into its own node list (DFS pre-order, left first).
struct RefSub {
  std::vector<RefTmpNode> nodes;
};

class RefBuilder {
 public:
  RefBuilder(const RefCtx& c, uint32_t nv) : c_(c), stamp_(nv, 0) {}

  // Splits ``idx`` per KDTree::splitBest (KDTree.cpp:129-228). Returns true and fills
  // L, R when the node splits; false for a leaf. Always fills the node box.
  bool split(const std::vector<uint32_t>& idx, float mn[3], float mx[3], std::vector<uint32_t>& L,
             std::vector<uint32_t>& R) {
    const float* V = c_.v;
    const uint32_t* T = c_.t;
    // box from the first triangle's first vertex, then all vertices (KDTree.cpp:139-153)
    const float* p0 = V + 3 * (size_t)T[3 * (size_t)idx[0]];
    for (int a = 0; a < 3; a++) mn[a] = mx[a] = p0[a];
    for (uint32_t tr : idx)
      for (int k = 0; k < 3; k++) {
        const float* p = V + 3 * (size_t)T[3 * (size_t)tr + k];
        for (int a = 0; a < 3; a++) {
          mn[a] = p[a] < mn[a] ? p[a] : mn[a];
          mx[a] = p[a] > mx[a] ? p[a] : mx[a];
        }
      }
    if (idx.size() <= 1) return false;  // maxLeafTriangleNum = 1
    float best_ratio = 10, best_split = 0;
    int best_dim = 0;
    int ndims = c_.policy == 0 ? 1 : 3;
    for (int dim = 0; dim < ndims; dim++) {
      cur_++;
      coords_.clear();
      for (uint32_t tr : idx)
        for (int k = 0; k < 3; k++) {
          uint32_t vi = T[3 * (size_t)tr + k];
          if (stamp_[vi] != cur_) {
            stamp_[vi] = cur_;
            coords_.push_back(V[3 * (size_t)vi + dim]);
          }
        }
      size_t mid = coords_.size() >> 1;
      std::nth_element(coords_.begin(), coords_.begin() + mid, coords_.end());
      float s = coords_[mid];
      unsigned left = 0;
      for (uint32_t tr : idx) {
        bool any = false;
        for (int k = 0; k < 3; k++) any |= V[3 * (size_t)T[3 * (size_t)tr + k] + dim] <= s;
        left += any;
      }
      float ratio = left / float(idx.size());
      bool better = c_.policy == 0 ? (dim == 0) : (std::fabs(ratio - 0.5) < std::fabs(best_ratio - 0.5));
      if (better) { best_ratio = ratio; best_dim = dim; best_split = s; }
    }
    if (best_ratio == 0 || best_ratio == 1) return false;
    L.clear();
    R.clear();
    for (uint32_t tr : idx) {
      bool any = false;
      for (int k = 0; k < 3; k++) any |= V[3 * (size_t)T[3 * (size_t)tr + k] + best_dim] <= best_split;
      (any ? L : R).push_back(tr);
    }
    return true;
  }

  // Builds a whole subtree into sub (DFS pre-order). Returns the local root id.
  int build(std::vector<uint32_t>& idx, int depth, RefSub& sub) {
    int id = (int)sub.nodes.size();
    sub.nodes.emplace_back();
    RefTmpNode n;
    std::vector<uint32_t> L, R;
    n.depth = depth;
    bool s = split(idx, n.mn, n.mx, L, R);
    if (!s) {
      n.leaf_tris.swap(idx);
      sub.nodes[id] = std::move(n);
      return id;
    }
    std::vector<uint32_t>().swap(idx);
    sub.nodes[id] = std::move(n);
    int l = build(L, depth + 1, sub);
    int r = build(R, depth + 1, sub);
    sub.nodes[id].left = l;
    sub.nodes[id].right = r;
    return id;
  }

 private:
  RefCtx c_;
  std::vector<uint32_t> stamp_;
  uint32_t cur_ = 0;
  std::vector<float> coords_;
};

}  // namespace

bool build_ref_order(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt, int policy, int threads,
                     RefOrder& out) {
  out = RefOrder();
  if (nt == 0) return false;
  RefCtx c{verts, tris, policy};
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());

  // Expand the top of the tree breadth-first on this thread until there are enough
  // independent subtrees, then build those in parallel; splicing keeps DFS order.
  struct Frontier {
    std::vector<uint32_t> idx;
    int depth;
    int slot;  // position in the top-level node list
  };
  std::vector<RefTmpNode> top;        // nodes expanded here (pre-order fixed later)
  std::vector<int> top_sub;           // for top nodes that are subtree roots: subtree id
  std::vector<Frontier> work;
  std::vector<uint32_t> all(nt);
  for (uint32_t i = 0; i < nt; i++) all[i] = i;
  RefBuilder rb(c, nv);

  // top-level node k has children ids into `top` or marks a deferred subtree
  top.emplace_back();
  top_sub.push_back(-1);
  std::vector<std::pair<std::vector<uint32_t>, int>> queue;  // (idx, top slot)
  queue.emplace_back(std::move(all), 0);
  std::vector<int> top_depth(1, 0);
  size_t target = (size_t)threads * 4;
  size_t head = 0;
  while (head < queue.size() && queue.size() - head < target && head < 4096) {
    int slot = queue[head].second;
    std::vector<uint32_t> idx = std::move(queue[head].first);
    int dep = top_depth[slot];
    RefTmpNode n;
    std::vector<uint32_t> L, R;
    bool s = rb.split(idx, n.mn, n.mx, L, R);
    n.depth = dep;
    if (!s) {
      n.leaf_tris.swap(idx);
      top[slot] = std::move(n);
    } else {
      int l = (int)top.size();
      int r = l + 1;
      n.left = l;
      n.right = r;
      top[slot] = std::move(n);
      top.emplace_back();
      top.emplace_back();
      top_sub.push_back(-1);
      top_sub.push_back(-1);
      top_depth.push_back(dep + 1);
      top_depth.push_back(dep + 1);
      queue.emplace_back(std::move(L), l);
      queue.emplace_back(std::move(R), r);
    }
    head++;
  }
  // remaining queue entries become parallel subtrees
  std::vector<RefSub> subs(queue.size() - head);
  std::vector<std::vector<uint32_t>> sub_idx(subs.size());
  std::vector<int> sub_slot(subs.size());
  for (size_t k = head; k < queue.size(); k++) {
    sub_idx[k - head] = std::move(queue[k].first);
    sub_slot[k - head] = queue[k].second;
    top_sub[queue[k].second] = (int)(k - head);
  }
  {
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    int nthr = (int)std::min<size_t>(threads, subs.size());
    for (int w = 0; w < nthr; w++)
      pool.emplace_back([&]() {
        RefBuilder local(c, nv);
        for (size_t k; (k = next.fetch_add(1)) < subs.size();)
          local.build(sub_idx[k], top_depth[sub_slot[k]], subs[k]);
      });
    for (auto& th : pool) th.join();
  }

  // Splice into one DFS pre-order list.
  out.nodes.reserve(top.size() + [&] { size_t s = 0; for (auto& x : subs) s += x.nodes.size(); return s; }());
  out.tri_order.reserve(nt);
  std::vector<std::vector<uint32_t>*> leaf_lists;
  struct Emit {
    RefOrder& o;
    std::vector<RefTmpNode>& top;
    std::vector<int>& top_sub;
    std::vector<RefSub>& subs;
    int emit_sub(RefSub& s, int li, int parent) {
      int id = (int)o.nodes.size();
      o.nodes.emplace_back();
      RefTmpNode& n = s.nodes[li];
      RefNodeHost h;
      std::memcpy(h.mn, n.mn, sizeof h.mn);
      std::memcpy(h.mx, n.mx, sizeof h.mx);
      h.parent = parent;
      h.left = h.right = -1;
      h.tri_begin = h.tri_end = 0;
      if (n.depth > o.max_depth) o.max_depth = n.depth;
      if (n.left < 0) {
        h.tri_begin = (uint32_t)o.tri_order.size();
        o.tri_order.insert(o.tri_order.end(), n.leaf_tris.begin(), n.leaf_tris.end());
        h.tri_end = (uint32_t)o.tri_order.size();
        o.nodes[id] = h;
        return id;
      }
      o.nodes[id] = h;
      int l = emit_sub(s, n.left, id);
      int r = emit_sub(s, n.right, id);
      o.nodes[id].left = l;
      o.nodes[id].right = r;
      return id;
    }
    int emit_top(int ti, int parent) {
      if (top_sub[ti] >= 0) return emit_sub(subs[top_sub[ti]], 0, parent);
      int id = (int)o.nodes.size();
      o.nodes.emplace_back();
      RefTmpNode& n = top[ti];
      RefNodeHost h;
      std::memcpy(h.mn, n.mn, sizeof h.mn);
      std::memcpy(h.mx, n.mx, sizeof h.mx);
      h.parent = parent;
      h.left = h.right = -1;
      h.tri_begin = h.tri_end = 0;
      if (n.depth > o.max_depth) o.max_depth = n.depth;
      if (n.left < 0) {
        h.tri_begin = (uint32_t)o.tri_order.size();
        o.tri_order.insert(o.tri_order.end(), n.leaf_tris.begin(), n.leaf_tris.end());
        h.tri_end = (uint32_t)o.tri_order.size();
        o.nodes[id] = h;
        return id;
      }
      o.nodes[id] = h;
      int l = emit_top(n.left, id);
      int r = emit_top(n.right, id);
      o.nodes[id].left = l;
      o.nodes[id].right = r;
      return id;
    }
  } em{out, top, top_sub, subs};
  em.emit_top(0, -1);

  out.tri_leaf.assign(nt, 0);
  out.tri_pos.assign(nt, 0);
  for (size_t i = 0; i < out.nodes.size(); i++) {
    const RefNodeHost& n = out.nodes[i];
    if (n.left >= 0) continue;
    uint32_t leaf = (uint32_t)out.leaf_node.size();
    out.leaf_node.push_back((uint32_t)i);
    for (uint32_t k = n.tri_begin; k < n.tri_end; k++) {
      out.tri_leaf[out.tri_order[k]] = leaf;
      out.tri_pos[out.tri_order[k]] = k;
    }
  }
  return true;
}

// ----------------------------------------------------------------------------------
// Binned SAH BVH
// ----------------------------------------------------------------------------------
namespace {

struct Aabb {
  float lo[3] = {INFINITY, INFINITY, INFINITY};
  float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  void grow(const Aabb& b) {
    for (int a = 0; a < 3; a++) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); }
  }
  void grow(const float* p) {
    for (int a = 0; a < 3; a++) { lo[a] = std::min(lo[a], p[a]); hi[a] = std::max(hi[a], p[a]); }
  }
  float area() const {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (dx < 0 || dy < 0 || dz < 0) return 0;
    return 2 * (dx * dy + dy * dz + dz * dx);
  }
};

constexpr int kBins = 16;
constexpr int kMaxLeaf = 8;
constexpr int kSahDepth = 40;  // beyond this depth, median splits bound the total depth

struct BvhBuilder {
  const std::vector<Aabb>& tb;      // per-triangle boxes
  const std::vector<float>& cen;    // centroids, 3 per triangle
  std::vector<uint32_t>& idx;
  std::vector<BvhNodeHost>& nodes;
  std::atomic<int>& node_count;
  std::atomic<int>& max_depth;
  int leaf_size;
  float pad;

  Aabb bounds(uint32_t b, uint32_t e) const {
    Aabb r;
    for (uint32_t i = b; i < e; i++) r.grow(tb[idx[i]]);
    return r;
  }

  void padded(const Aabb& a, float lo[3], float hi[3]) const {
    for (int k = 0; k < 3; k++) {
      lo[k] = a.lo[k] - pad - std::fabs(a.lo[k]) * 1e-6f;
      hi[k] = a.hi[k] + pad + std::fabs(a.hi[k]) * 1e-6f;
    }
  }

  // Splits [b,e); returns the split point m (b < m < e).
  uint32_t split(uint32_t b, uint32_t e, int depth, bool& make_leaf) {
    uint32_t n = e - b;
    make_leaf = false;
    Aabb cb;
    for (uint32_t i = b; i < e; i++) cb.grow(&cen[3 * (size_t)idx[i]]);
    int axis = 0;
    float ext = -1;
    for (int a = 0; a < 3; a++)
      if (cb.hi[a] - cb.lo[a] > ext) { ext = cb.hi[a] - cb.lo[a]; axis = a; }
    if (ext <= 0) {  // all centroids coincide
      if ((int)n <= kMaxLeaf) { make_leaf = true; return b; }
      return b + n / 2;
    }
    if (depth >= kSahDepth) {
      uint32_t m = b + n / 2;
      std::nth_element(idx.begin() + b, idx.begin() + m, idx.begin() + e, [&](uint32_t x, uint32_t y) {
        return cen[3 * (size_t)x + axis] < cen[3 * (size_t)y + axis];
      });
      return m;
    }
    float best_cost = INFINITY;
    int best_axis = -1, best_bin = -1;
    for (int a = 0; a < 3; a++) {
      float lo = cb.lo[a], w = cb.hi[a] - cb.lo[a];
      if (w <= 0) continue;
      Aabb bb[kBins];
      int cnt[kBins] = {0};
      float s = kBins / w;
      for (uint32_t i = b; i < e; i++) {
        uint32_t t = idx[i];
        int k = std::min(kBins - 1, (int)((cen[3 * (size_t)t + a] - lo) * s));
        cnt[k]++;
        bb[k].grow(tb[t]);
      }
      float right_area[kBins];
      int right_cnt[kBins];
      Aabb acc;
      int ac = 0;
      for (int k = kBins - 1; k > 0; k--) {
        acc.grow(bb[k]);
        ac += cnt[k];
        right_area[k] = acc.area();
        right_cnt[k] = ac;
      }
      acc = Aabb();
      ac = 0;
      for (int k = 0; k < kBins - 1; k++) {
        acc.grow(bb[k]);
        ac += cnt[k];
        if (ac == 0 || right_cnt[k + 1] == 0) continue;
        float cost = acc.area() * ac + right_area[k + 1] * right_cnt[k + 1];
        if (cost < best_cost) { best_cost = cost; best_axis = a; best_bin = k; }
      }
    }
    Aabb nb = bounds(b, e);
    float leaf_cost = nb.area() * n;
    if (best_axis < 0 || (best_cost >= leaf_cost && (int)n <= kMaxLeaf)) {
      if ((int)n <= kMaxLeaf) { make_leaf = true; return b; }
      if (best_axis < 0) return b + n / 2;
    }
    float lo = cb.lo[best_axis], s = kBins / (cb.hi[best_axis] - cb.lo[best_axis]);
    auto it = std::partition(idx.begin() + b, idx.begin() + e, [&](uint32_t t) {
      int k = std::min(kBins - 1, (int)((cen[3 * (size_t)t + best_axis] - lo) * s));
      return k <= best_bin;
    });
    uint32_t m = (uint32_t)(it - idx.begin());
    if (m == b || m == e) m = b + n / 2;
    return m;
  }

  // Builds the subtree for [b,e) whose box is `box`; returns the child reference
  // (inner node id, or ~slot for a leaf) and the leaf count through cnt.
  int32_t build(uint32_t b, uint32_t e, int depth, int32_t& cnt, bool parallel) {
    int d = max_depth.load();
    while (depth > d && !max_depth.compare_exchange_weak(d, depth)) {}
    uint32_t n = e - b;
    if ((int)n <= leaf_size) { cnt = (int32_t)n; return ~(int32_t)b; }
    bool leaf = false;
    uint32_t m = split(b, e, depth, leaf);
    if (leaf) { cnt = (int32_t)n; return ~(int32_t)b; }
    int id = node_count.fetch_add(1);
    BvhNodeHost& nd = nodes[id];
    padded(bounds(b, m), nd.c0lo, nd.c0hi);
    padded(bounds(m, e), nd.c1lo, nd.c1hi);
    int32_t c0, c1, n0 = 0, n1 = 0;
    if (parallel && n > 65536) {
      std::thread th([&] { c0 = build(b, m, depth + 1, n0, true); });
      c1 = build(m, e, depth + 1, n1, true);
      th.join();
    } else {
      c0 = build(b, m, depth + 1, n0, false);
      c1 = build(m, e, depth + 1, n1, false);
    }
    nodes[id].child[0] = c0;
    nodes[id].child[1] = c1;
    nodes[id].count[0] = c0 < 0 ? n0 : 0;
    nodes[id].count[1] = c1 < 0 ? n1 : 0;
    return id;
  }
};

}  // namespace

bool build_bvh(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt, int leaf_size, int threads,
               Bvh& out) {
  (void)threads;
  out = Bvh();
  if (nt == 0) return false;
  leaf_size = std::max(1, std::min(leaf_size, kMaxLeaf));
  std::vector<Aabb> tb(nt);
  std::vector<float> cen(3 * (size_t)nt);
  float scene_max = 0;
  for (uint32_t t = 0; t < nt; t++) {
    for (int k = 0; k < 3; k++) tb[t].grow(verts + 3 * (size_t)tris[3 * (size_t)t + k]);
    for (int a = 0; a < 3; a++) {
      cen[3 * (size_t)t + a] = 0.5f * (tb[t].lo[a] + tb[t].hi[a]);
      scene_max = std::max(scene_max, std::max(std::fabs(tb[t].lo[a]), std::fabs(tb[t].hi[a])));
    }
  }
  (void)nv;
  out.tri_order.resize(nt);
  for (uint32_t i = 0; i < nt; i++) out.tri_order[i] = i;
  out.nodes.resize(std::max<uint32_t>(1, nt));
  std::atomic<int> count{0}, depth{0};
  BvhBuilder bb{tb, cen, out.tri_order, out.nodes, count, depth, leaf_size, 1e-5f * (1.0f + scene_max)};
  int32_t cnt = 0;
  if (nt <= (uint32_t)leaf_size) {
    // a root whose two children are the one leaf and a copy of its first triangle
    // (re-testing a triangle never changes the answer)
    BvhNodeHost& r = out.nodes[0];
    count = 1;
    bb.padded(bb.bounds(0, nt), r.c0lo, r.c0hi);
    bb.padded(bb.bounds(0, 1), r.c1lo, r.c1hi);
    r.child[0] = ~0;
    r.count[0] = (int32_t)nt;
    r.child[1] = ~0;
    r.count[1] = 1;
  } else {
    int32_t root = bb.build(0, nt, 0, cnt, true);
    (void)root;  // root is node 0: the first node allocated
  }
  out.nodes.resize(count.load());
  out.max_depth = depth.load();
  out.leaf_size = leaf_size;
  return true;
}

}  // namespace rx

// ----------------------------------------------------------------------------------
// C ABI: host-only serialization of the reference-order tree
// ----------------------------------------------------------------------------------
#include "../../include/renderx.h"

extern "C" rx_status rx_reftree_serialize(const float* verts, uint32_t nv, const uint32_t* tris, uint32_t nt,
                                          int32_t policy, float* nodes12, uint32_t* num_nodes, float* leaf_tid,
                                          uint32_t* num_leaf_tris) {
  if (!verts || !tris || !num_nodes || !num_leaf_tris || nt == 0 || nv == 0) return RX_ERR_INVALID;
  if (policy != 0 && policy != 1) return RX_ERR_INVALID;
  for (size_t k = 0; k < 3 * (size_t)nt; k++)
    if (tris[k] >= nv) return RX_ERR_INVALID;
  rx::RefOrder ro;
  if (!rx::build_ref_order(verts, nv, tris, nt, policy, 0, ro)) return RX_ERR_INVALID;
  uint32_t cap_n = *num_nodes, cap_l = *num_leaf_tris;
  *num_nodes = (uint32_t)ro.nodes.size();
  *num_leaf_tris = (uint32_t)ro.tri_order.size();
  if (!nodes12 || !leaf_tid) return RX_OK;
  if (cap_n < ro.nodes.size() || cap_l < ro.tri_order.size()) return RX_ERR_INVALID;
  for (size_t i = 0; i < ro.nodes.size(); i++) {
    const rx::RefNodeHost& n = ro.nodes[i];
    float* o = nodes12 + 12 * i;
    o[0] = (float)n.parent;
    if (n.left >= 0) { o[1] = (float)n.right; o[2] = -1; o[3] = -1; }
    else { o[1] = -1; o[2] = (float)n.tri_begin; o[3] = (float)n.tri_end; }
    o[4] = n.mn[0]; o[5] = n.mn[1]; o[6] = n.mn[2]; o[7] = 0;
    o[8] = n.mx[0]; o[9] = n.mx[1]; o[10] = n.mx[2]; o[11] = 0;
  }
  for (size_t k = 0; k < ro.tri_order.size(); k++) leaf_tid[k] = (float)ro.tri_order[k];
  return RX_OK;
}

namespace rx {

namespace {
struct Child4 {
  int32_t ref, count;
  float lo[3], hi[3];
};
float half_area(const Child4& c) {
  float ex = c.hi[0] - c.lo[0], ey = c.hi[1] - c.lo[1], ez = c.hi[2] - c.lo[2];
  return ex * ey + ey * ez + ez * ex;
}
void children_of(const BvhNodeHost& n, Child4 (&c)[2]) {
  for (int k = 0; k < 3; k++) {
    c[0].lo[k] = n.c0lo[k];
    c[0].hi[k] = n.c0hi[k];
    c[1].lo[k] = n.c1lo[k];
    c[1].hi[k] = n.c1hi[k];
  }
  c[0].ref = n.child[0];
  c[0].count = n.count[0];
  c[1].ref = n.child[1];
  c[1].count = n.count[1];
}
// One node of a W-wide BVH from binary node n2: its children opened largest surface area
// first until W of them; node layout: per axis the W lower then the W upper child bounds,
// then W refs and W leaf counts (8 W floats).
template <int W>
int32_t collapse(const Bvh& b2, int32_t n2, int depth, Bvh4& out) {
  Child4 two[2];
  children_of(b2.nodes[n2], two);
  std::vector<Child4> kids = {two[0], two[1]};
  while (kids.size() < (size_t)W) {
    int best = -1;
    float area = -1.0f;
    for (size_t i = 0; i < kids.size(); i++)
      if (kids[i].ref >= 0 && half_area(kids[i]) > area) area = half_area(kids[i]), best = (int)i;
    if (best < 0) break;
    Child4 sub[2];
    children_of(b2.nodes[kids[best].ref], sub);
    kids[best] = sub[0];
    kids.push_back(sub[1]);
  }
  constexpr int kF = 8 * W;  // floats per node
  const int32_t me = (int32_t)(out.data.size() / kF);
  out.data.resize(out.data.size() + kF, 0.0f);
  out.max_depth = std::max(out.max_depth, depth);
  int32_t refs[W];
  for (int j = 0; j < W; j++) refs[j] = kBvh4Empty;
  for (size_t j = 0; j < kids.size(); j++)  // inner node index, or the leaf packed with its count
    refs[j] = kids[j].ref >= 0 ? collapse<W>(b2, kids[j].ref, depth + 1, out) : pack_leaf(~kids[j].ref, kids[j].count);
  float* f = out.data.data() + kF * (size_t)me;  // after the recursion: data may have moved
  for (int j = 0; j < W; j++) {
    bool has = j < (int)kids.size();
    for (int k = 0; k < 3; k++) {  // an empty slot is an inverted box: no ray enters it
      f[2 * W * k + j] = has ? kids[j].lo[k] : INFINITY;
      f[2 * W * k + W + j] = has ? kids[j].hi[k] : -INFINITY;
    }
    std::memcpy(&f[6 * W + j], &refs[j], 4);  // f[7 W + j]: spare, zero
  }
  return me;
}
}  // namespace

void collapse_bvh4(const Bvh& b2, Bvh4& out) {
  out.data.clear();
  out.max_depth = 0;
  if (!b2.nodes.empty()) collapse<4>(b2, 0, 0, out);
}

void collapse_bvh8(const Bvh& b2, Bvh4& out) {
  out.data.clear();
  out.max_depth = 0;
  if (!b2.nodes.empty()) collapse<8>(b2, 0, 0, out);
}

}  // namespace rx
