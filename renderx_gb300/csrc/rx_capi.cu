// The C ABI (include/renderx.h): context, scene upload, accelerator build and the
// closest-hit entry points.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "rx_guide.h"
#include "rx_internal.h"

using rx::DevBuf;
using rx::DeviceGuard;

namespace {

rx_status upload(rx_context* c, DevBuf& b, const void* src, size_t bytes, const char* what) {
  rx_status s = c->cuda(b.alloc(bytes), what);
  if (s != RX_OK || bytes == 0) return s;
  return c->cuda(cudaMemcpy(b.p, src, bytes, cudaMemcpyHostToDevice), what);
}

}  // namespace

extern "C" {

const char* rx_version(void) { return "renderx_gb300 0.1 (sm_103a)"; }

rx_status rx_create(rx_context** out, int device) {
  if (!out) return RX_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return RX_ERR_CUDA;
  if (device < 0 || device >= ndev) return RX_ERR_INVALID;
  rx_context* c = new (std::nothrow) rx_context();
  if (!c) return RX_ERR_OOM;
  c->device = device;
  DeviceGuard g(device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->copy_stream[0], cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->copy_stream[1], cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return RX_ERR_CUDA;
  }
  if (c->d_counters.alloc(64 * sizeof(unsigned long long)) != cudaSuccess) {
    delete c;
    return RX_ERR_OOM;
  }
  cudaMemset(c->d_counters.p, 0, c->d_counters.bytes);
  cudaDeviceGetAttribute(&c->trace_cfg.sms, cudaDevAttrMultiProcessorCount, device);
  *out = c;
  return RX_OK;
}

void rx_destroy(rx_context* c) {
  if (!c) return;
  {
    DeviceGuard g(c->device);
    cudaDeviceSynchronize();
    for (DevBuf* b : {&c->d_bvh, &c->d_bvh4, &c->d_bvh8, &c->d_tris, &c->d_tri_nrm, &c->d_ref, &c->d_ref_leaf_node, &c->d_ref_leaf_range, &c->d_ref_tris,
                      &c->d_anc_range, &c->d_anc_nodes, &c->d_anc_box, &c->d_slot_n, &c->d_tri_v, &c->d_tri_n, &c->d_tri_obj,
                      &c->d_objects, &c->d_light_cdf, &c->d_light_tri,
                      &c->d_counters, &c->d_queue})
      b->release();
    for (int k = 0; k < rx_context::kRing; k++) {
      for (DevBuf* b : {&c->ring_rays[k], &c->ring_tid[k], &c->ring_dist[k], &c->ring_queue[k], &c->ring_counters[k]})
        b->release();
      for (cudaEvent_t& e : c->ring_ev[k])
        if (e) cudaEventDestroy(e);
      if (c->ring_stream[k]) cudaStreamDestroy(c->ring_stream[k]);
    }
    for (cudaEvent_t e : c->timing_ev) cudaEventDestroy(e);
    rx::guide_free(c->guide);
    c->guide = nullptr;
    if (c->stream) cudaStreamDestroy(c->stream);
    for (auto s : c->copy_stream)
      if (s) cudaStreamDestroy(s);
  }
  delete c;
}

const char* rx_last_error(const rx_context* c) { return c ? c->err.c_str() : "null context"; }

rx_status rx_scene_set_geometry(rx_context* c, const float* verts, uint32_t nv, const uint32_t* tri_vidx, uint32_t nt,
                                const uint32_t* tri_obj, const uint32_t* tri_local, const float* vnormals) {
  if (!c) return RX_ERR_INVALID;
  if (!verts || !tri_vidx || nv == 0 || nt == 0) return c->fail(RX_ERR_INVALID, "empty geometry");
  for (size_t k = 0; k < 3 * (size_t)nt; k++)
    if (tri_vidx[k] >= nv) return c->fail(RX_ERR_INVALID, "triangle vertex index out of range");
  for (size_t k = 0; k < 3 * (size_t)nv; k++)
    if (!std::isfinite(verts[k])) return c->fail(RX_ERR_INVALID, "non-finite vertex coordinate");
  c->verts.assign(verts, verts + 3 * (size_t)nv);
  c->tris.assign(tri_vidx, tri_vidx + 3 * (size_t)nt);
  c->tri_obj.assign(nt, 0);
  c->tri_local.resize(nt);
  for (uint32_t i = 0; i < nt; i++) c->tri_local[i] = i;
  if (tri_obj) c->tri_obj.assign(tri_obj, tri_obj + nt);
  if (tri_local) c->tri_local.assign(tri_local, tri_local + nt);
  c->has_normals = vnormals != nullptr;
  if (vnormals) c->vnormals.assign(vnormals, vnormals + 3 * (size_t)nv);
  else c->vnormals.clear();
  c->geometry_dirty = true;
  c->accel_ready = false;
  return RX_OK;
}

rx_status rx_scene_set_objects(rx_context* c, const rx_object* objs, uint32_t nobj) {
  if (!c) return RX_ERR_INVALID;
  if (nobj && !objs) return c->fail(RX_ERR_INVALID, "null objects");
  c->objects.assign(objs, objs + nobj);
  return RX_OK;
}

rx_status rx_build_accel(rx_context* c, const rx_build_options* opts) {
  if (!c) return RX_ERR_INVALID;
  if (c->tris.empty()) return c->fail(RX_ERR_STATE, "no geometry");
  rx_build_options o{0, 0, 0, 0};
  if (opts) o = *opts;
  if (o.split_policy != 0 && o.split_policy != 1) return c->fail(RX_ERR_INVALID, "split_policy must be 0 or 1");
  if (o.leaf_size <= 0) o.leaf_size = 3;
  if (o.leaf_size > 8) return c->fail(RX_ERR_INVALID, "leaf_size must be 1..8");
  uint32_t nv = (uint32_t)(c->verts.size() / 3), nt = (uint32_t)(c->tris.size() / 3);
  if (nt >= (1u << 28)) return c->fail(RX_ERR_UNSUPPORTED, "at most 2^28 - 1 triangles (packed leaf refs)");
  if (!rx::build_ref_order(c->verts.data(), nv, c->tris.data(), nt, o.split_policy, o.host_threads, c->ref))
    return c->fail(RX_ERR_INVALID, "reference-order build failed");
  if (!rx::build_bvh(c->verts.data(), nv, c->tris.data(), nt, o.leaf_size, o.host_threads, c->bvh))
    return c->fail(RX_ERR_INVALID, "BVH build failed");
  if (c->bvh.max_depth >= rx::kStackDepth) return c->fail(RX_ERR_UNSUPPORTED, "BVH deeper than the traversal stack");

  DeviceGuard g(c->device);
  // BVH nodes: 4 float4 each
  std::vector<float4> nodes(4 * c->bvh.nodes.size());
  for (size_t i = 0; i < c->bvh.nodes.size(); i++) {
    const rx::BvhNodeHost& h = c->bvh.nodes[i];
    nodes[4 * i + 0] = make_float4(h.c0lo[0], h.c0hi[0], h.c0lo[1], h.c0hi[1]);
    nodes[4 * i + 1] = make_float4(h.c1lo[0], h.c1hi[0], h.c1lo[1], h.c1hi[1]);
    nodes[4 * i + 2] = make_float4(h.c0lo[2], h.c0hi[2], h.c1lo[2], h.c1hi[2]);
    float4 l;
    std::memcpy(&l.x, &h.child[0], 4);
    std::memcpy(&l.y, &h.child[1], 4);
    std::memcpy(&l.z, &h.count[0], 4);
    std::memcpy(&l.w, &h.count[1], 4);
    nodes[4 * i + 3] = l;
  }
  auto bits = [](uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
  };
  const float* V = c->verts.data();
  auto vtx = [&](uint32_t t, int k, uint32_t w) {
    const float* p = V + 3 * (size_t)c->tris[3 * (size_t)t + k];
    return make_float4(p[0], p[1], p[2], bits(w));
  };
  std::vector<float4> slots(3 * (size_t)nt);
  for (uint32_t s = 0; s < nt; s++) {
    uint32_t t = c->bvh.tri_order[s];
    slots[3 * (size_t)s + 0] = vtx(t, 0, t);
    slots[3 * (size_t)s + 1] = vtx(t, 1, c->ref.tri_leaf[t]);
    slots[3 * (size_t)s + 2] = vtx(t, 2, c->ref.tri_pos[t]);
  }
  // reference nodes: (min, parent), (max, right child or ~leaf index)
  std::vector<float4> refn(2 * c->ref.nodes.size());
  std::vector<int32_t> node_leaf(c->ref.nodes.size(), -1);
  for (size_t l = 0; l < c->ref.leaf_node.size(); l++) node_leaf[c->ref.leaf_node[l]] = (int32_t)l;
  std::vector<uint32_t> leaf_range(2 * c->ref.leaf_node.size());
  for (size_t i = 0; i < c->ref.nodes.size(); i++) {
    const rx::RefNodeHost& h = c->ref.nodes[i];
    int32_t w = h.left >= 0 ? h.right : ~node_leaf[i];
    refn[2 * i] = make_float4(h.mn[0], h.mn[1], h.mn[2], bits((uint32_t)h.parent));
    refn[2 * i + 1] = make_float4(h.mx[0], h.mx[1], h.mx[2], bits((uint32_t)w));
    if (h.left < 0) {
      leaf_range[2 * node_leaf[i]] = h.tri_begin;
      leaf_range[2 * node_leaf[i] + 1] = h.tri_end;
    }
  }
  std::vector<float4> reft(3 * (size_t)nt);
  for (uint32_t k = 0; k < nt; k++) {
    uint32_t t = c->ref.tri_order[k];
    reft[3 * (size_t)k] = vtx(t, 0, t);
    reft[3 * (size_t)k + 1] = vtx(t, 1, 0);
    reft[3 * (size_t)k + 2] = vtx(t, 2, 0);
  }
  std::vector<int32_t> leaf_node(c->ref.leaf_node.begin(), c->ref.leaf_node.end());
  // per reference leaf, the node ids of its root path (leaf first): the boxes the
  // reference tests before it reaches the leaf's triangles
  std::vector<uint32_t> anc_range(2 * leaf_node.size());
  std::vector<int32_t> anc_nodes;
  anc_nodes.reserve(leaf_node.size() * (size_t)(c->ref.max_depth + 1));
  for (size_t l = 0; l < leaf_node.size(); l++) {
    anc_range[2 * l] = (uint32_t)anc_nodes.size();
    for (int32_t nd = leaf_node[l]; nd >= 0; nd = c->ref.nodes[nd].parent) anc_nodes.push_back(nd);
    anc_range[2 * l + 1] = (uint32_t)anc_nodes.size();
  }
  // the same root paths as boxes, contiguous per leaf (one dependent load fewer)
  std::vector<float4> anc_box(2 * anc_nodes.size());
  for (size_t k = 0; k < anc_nodes.size(); k++) {
    anc_box[2 * k] = refn[2 * (size_t)anc_nodes[k]];
    anc_box[2 * k + 1] = refn[2 * (size_t)anc_nodes[k] + 1];
  }
  rx_status s;
  if ((s = upload(c, c->d_bvh, nodes.data(), nodes.size() * sizeof(float4), "upload BVH")) != RX_OK) return s;
  rx::collapse_bvh4(c->bvh, c->bvh4);
  if ((s = upload(c, c->d_bvh4, c->bvh4.data.data(), c->bvh4.data.size() * sizeof(float), "upload BVH4")) != RX_OK)
    return s;
  rx::collapse_bvh8(c->bvh, c->bvh8);
  if ((s = upload(c, c->d_bvh8, c->bvh8.data.data(), c->bvh8.data.size() * sizeof(float), "upload BVH8")) != RX_OK)
    return s;
  if ((s = upload(c, c->d_tris, slots.data(), slots.size() * sizeof(float4), "upload triangles")) != RX_OK) return s;
  const uint32_t nslots = (uint32_t)(slots.size() / 3);
  if ((s = c->cuda(c->d_tri_nrm.alloc((size_t)std::max<uint32_t>(nslots, 1) * sizeof(float4)), "triangle normals")) !=
      RX_OK)
    return s;
  if ((s = c->cuda(rx::launch_slot_normals(c->d_tris.as<float4>(), nslots, c->d_tri_nrm.as<float4>(), c->stream),
                   "triangle normals")) != RX_OK)
    return s;
  // traces may follow on any stream
  if ((s = c->cuda(cudaStreamSynchronize(c->stream), "triangle normals")) != RX_OK) return s;
  if ((s = upload(c, c->d_ref, refn.data(), refn.size() * sizeof(float4), "upload reference nodes")) != RX_OK) return s;
  if ((s = upload(c, c->d_ref_leaf_node, leaf_node.data(), leaf_node.size() * 4, "upload leaf map")) != RX_OK) return s;
  if ((s = upload(c, c->d_ref_leaf_range, leaf_range.data(), leaf_range.size() * 4, "upload leaf ranges")) != RX_OK)
    return s;
  if ((s = upload(c, c->d_ref_tris, reft.data(), reft.size() * sizeof(float4), "upload reference triangles")) != RX_OK)
    return s;
  if ((s = upload(c, c->d_anc_range, anc_range.data(), anc_range.size() * 4, "upload ancestor ranges")) != RX_OK)
    return s;
  if ((s = upload(c, c->d_anc_nodes, anc_nodes.data(), anc_nodes.size() * 4, "upload ancestor lists")) != RX_OK)
    return s;
  if ((s = upload(c, c->d_anc_box, anc_box.data(), anc_box.size() * sizeof(float4), "upload ancestor boxes")) != RX_OK)
    return s;
  rx::DevAccel& A = c->accel;
  A.bvh = c->d_bvh.as<float4>();
  A.tris = c->d_tris.as<float4>();
  A.tri_nrm = c->d_tri_nrm.as<float4>();
  A.ref = c->d_ref.as<float4>();
  A.ref_leaf_node = c->d_ref_leaf_node.as<int32_t>();
  A.ref_leaf_range = c->d_ref_leaf_range.as<uint32_t>();
  A.ref_tris = c->d_ref_tris.as<float4>();
  A.anc_range = c->d_anc_range.as<uint32_t>();
  A.anc_nodes = c->d_anc_nodes.as<int32_t>();
  A.anc_box = c->d_anc_box.as<float4>();
  A.num_nodes = (uint32_t)c->bvh.nodes.size();
  A.num_tris = nt;
  A.num_ref_nodes = (uint32_t)c->ref.nodes.size();
  A.num_ref_leaves = (uint32_t)c->ref.leaf_node.size();
  A.prune_rel = 1e-3f;
  A.bvh_depth = (uint32_t)c->bvh.max_depth;
  A.bvh4 = c->d_bvh4.as<float4>();
  A.bvh4_depth = (uint32_t)c->bvh4.max_depth;
  A.bvh8 = c->d_bvh8.as<float4>();
  A.bvh8_depth = (uint32_t)c->bvh8.max_depth;
  for (int k = 0; k < 3; k++) {
    const rx::BvhNodeHost& r = c->bvh.nodes[0];
    A.lo[k] = std::min(r.c0lo[k], r.c1lo[k]);
    A.hi[k] = std::max(r.c0hi[k], r.c1hi[k]);
  }
  c->accel_ready = true;
  c->geometry_dirty = false;
  if (!c->objects.empty()) return c->build_scene();
  return RX_OK;
}

}  // extern "C"

// Shading data for the light-transport kernels: objects, per-triangle vertices and
// normals (vertex normals where the object has them, else the face normal), the same
// normals in BVH slot order for the traversal's self-intersection condition, and the
// emitter sampler (cumulative triangle areas over the emissive objects, the product of
// Scene::SurfaceSampler's object choice and SceneObject::emit's triangle choice).
rx_status rx_context::build_scene() {
  rx_context* c = this;
  uint32_t nt = (uint32_t)(c->tris.size() / 3), nobj = (uint32_t)c->objects.size();
  for (uint32_t i = 0; i < nt; i++)
    if (c->tri_obj[i] >= nobj) return c->fail(RX_ERR_INVALID, "triangle object id out of range");
  for (uint32_t o = 0; o < nobj; o++)
    if (c->objects[o].material > RX_MAT_VPM) return c->fail(RX_ERR_INVALID, "unknown material");
  const float* V = c->verts.data();
  auto vtx = [&](uint32_t t, int k) {
    const float* p = V + 3 * (size_t)c->tris[3 * (size_t)t + k];
    return make_float4(p[0], p[1], p[2], 0.0f);
  };
  std::vector<float4> tv(3 * (size_t)nt), tn(3 * (size_t)nt), sn(3 * (size_t)nt);
  for (uint32_t t = 0; t < nt; t++) {
    float4 a = vtx(t, 0), b = vtx(t, 1), d = vtx(t, 2);
    tv[3 * (size_t)t] = a;
    tv[3 * (size_t)t + 1] = b;
    tv[3 * (size_t)t + 2] = d;
    bool vn = c->has_normals && c->objects[c->tri_obj[t]].has_vertex_normals;
    float e1[3] = {b.x - a.x, b.y - a.y, b.z - a.z}, e2[3] = {d.x - a.x, d.y - a.y, d.z - a.z};
    float fn[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    float l = std::sqrt(fn[0] * fn[0] + fn[1] * fn[1] + fn[2] * fn[2]);
    if (l > 0) for (float& x : fn) x /= l;
    for (int k = 0; k < 3; k++) {
      if (vn) {
        const float* q = c->vnormals.data() + 3 * (size_t)c->tris[3 * (size_t)t + k];
        tn[3 * (size_t)t + k] = make_float4(q[0], q[1], q[2], 0.0f);
      } else {
        tn[3 * (size_t)t + k] = make_float4(fn[0], fn[1], fn[2], 0.0f);
      }
    }
  }
  for (uint32_t s = 0; s < nt; s++) {
    uint32_t t = c->bvh.tri_order[s];
    for (int k = 0; k < 3; k++) sn[3 * (size_t)s + k] = tn[3 * (size_t)t + k];
    uint32_t ob = c->tri_obj[t];
    std::memcpy(&sn[3 * (size_t)s].w, &ob, 4);
  }
  std::vector<rx::DevObject> objs(nobj);
  std::vector<float> cdf;
  std::vector<uint32_t> ltri;
  double acc = 0;
  for (uint32_t o = 0; o < nobj; o++) {
    const rx_object& r = c->objects[o];
    rx::DevObject& d = objs[o];
    d.material = r.material;
    d.has_normals = (c->has_normals && r.has_vertex_normals) ? 1 : 0;
    d.tri_begin = r.tri_begin;
    d.tri_count = r.tri_count;
    std::memcpy(d.color, r.color, sizeof d.color);
    d.coeff = r.coeff;
    std::memcpy(d.diffuse_color, r.diffuse_color, sizeof d.diffuse_color);
    d.ior = r.ior;
    std::memcpy(d.sigma_s, r.sigma_s, sizeof d.sigma_s);
    std::memcpy(d.sigma_a, r.sigma_a, sizeof d.sigma_a);
    d.g = r.g;
    std::memcpy(d.decay, r.decay, sizeof d.decay);
    d.step_size = r.step_size > 0.0f ? r.step_size : 0.0005f;  // SceneVPMObject.h:64
  }
  for (uint32_t t = 0; t < nt; t++) {
    if (c->objects[c->tri_obj[t]].material != RX_MAT_EMISSIVE) continue;
    float4 a = tv[3 * (size_t)t], b = tv[3 * (size_t)t + 1], d = tv[3 * (size_t)t + 2];
    // SimpleShape::getTriangleArea: |(v1-v0) x (v2-v1)| / 2
    double l0[3] = {b.x - a.x, b.y - a.y, b.z - a.z}, l1[3] = {d.x - b.x, d.y - b.y, d.z - b.z};
    double cx = l0[1] * l1[2] - l0[2] * l1[1], cy = l0[2] * l1[0] - l0[0] * l1[2], cz = l0[0] * l1[1] - l0[1] * l1[0];
    acc += 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
    cdf.push_back((float)acc);
    ltri.push_back(t);
  }
  DeviceGuard g(c->device);
  rx_status st;
  if ((st = upload(c, c->d_tri_v, tv.data(), tv.size() * sizeof(float4), "upload triangle vertices")) != RX_OK) return st;
  if ((st = upload(c, c->d_tri_n, tn.data(), tn.size() * sizeof(float4), "upload triangle normals")) != RX_OK) return st;
  if ((st = upload(c, c->d_slot_n, sn.data(), sn.size() * sizeof(float4), "upload slot normals")) != RX_OK) return st;
  if ((st = upload(c, c->d_tri_obj, c->tri_obj.data(), nt * 4, "upload triangle objects")) != RX_OK) return st;
  if ((st = upload(c, c->d_objects, objs.data(), objs.size() * sizeof(rx::DevObject), "upload objects")) != RX_OK)
    return st;
  if (!cdf.empty()) {
    if ((st = upload(c, c->d_light_cdf, cdf.data(), cdf.size() * 4, "upload light cdf")) != RX_OK) return st;
    if ((st = upload(c, c->d_light_tri, ltri.data(), ltri.size() * 4, "upload light triangles")) != RX_OK) return st;
  }
  rx::DevScene& S = c->scene;
  S.accel = c->accel;
  S.slot_n = c->d_slot_n.as<float4>();
  S.tri_v = c->d_tri_v.as<float4>();
  S.tri_n = c->d_tri_n.as<float4>();
  S.tri_obj = c->d_tri_obj.as<uint32_t>();
  S.objects = c->d_objects.as<rx::DevObject>();
  S.num_objects = nobj;
  S.light_cdf = c->d_light_cdf.as<float>();
  S.light_tri = c->d_light_tri.as<uint32_t>();
  S.num_lights = (uint32_t)cdf.size();
  S.light_area = (float)acc;
  c->scene_ready = true;
  return RX_OK;
}

extern "C" {

rx_status rx_render_pt(rx_context* c, const rx_camera* cam, const rx_pt_options* opts, double* film_rgb,
                       double* film_sq, rx_render_stats* stats) {
  if (!c) return RX_ERR_INVALID;
  if (!cam || !opts || !film_rgb) return c->fail(RX_ERR_INVALID, "null argument");
  if (!c->scene_ready) return c->fail(RX_ERR_STATE, "scene objects not built (rx_scene_set_objects, rx_build_accel)");
  if (cam->width == 0 || cam->height == 0 || cam->sight_dist == 0) return c->fail(RX_ERR_INVALID, "bad camera");
  if (opts->spp == 0) return c->fail(RX_ERR_INVALID, "spp must be positive");
  if (opts->max_depth > 1000) return c->fail(RX_ERR_INVALID, "max_depth too large");
  if (opts->nee && c->scene.num_lights == 0) return c->fail(RX_ERR_INVALID, "light sampling needs an emissive object");
  if (opts->flags & ~RX_PT_GUIDED) return c->fail(RX_ERR_INVALID, "unknown flags");
  if (!(opts->time_budget_s >= 0.0f) || opts->reserved) return c->fail(RX_ERR_INVALID, "time_budget_s >= 0, reserved 0");
  if (opts->flags & RX_PT_GUIDED) {
    if (opts->nee) return c->fail(RX_ERR_INVALID, "guiding applies to PathTracer (nee = 0)");
    if (!rx::guide_ready(c->guide)) return c->fail(RX_ERR_STATE, "guided rendering needs rx_guide_init");
  }
  DeviceGuard g(c->device);
  size_t np = (size_t)cam->width * cam->height;
  DevBuf sum, sq;
  rx_status s;
  if ((s = c->cuda(sum.alloc(np * 3 * sizeof(double)), "film")) != RX_OK) return s;
  if (film_sq && (s = c->cuda(sq.alloc(np * 3 * sizeof(double)), "film")) != RX_OK) return s;
  cudaMemsetAsync(sum.p, 0, sum.bytes, c->stream);
  if (film_sq) cudaMemsetAsync(sq.p, 0, sq.bytes, c->stream);
  rx_render_stats st{};
  if ((s = c->cuda(rx::render_pt(c, *cam, *opts, sum.as<double>(), film_sq ? sq.as<double>() : nullptr, &st, c->stream),
                   "render_pt")) != RX_OK)
    return s;
  // paths run sample-major: with st.paths done, pixel q holds done / np samples, one
  // more when q < done % np (every pixel holds spp when the render completed)
  const uint64_t done = st.paths;
  auto count = [&](size_t q) { return (double)(done / np + (q < done % np ? 1 : 0)); };
  std::vector<double> h(np * 3);
  if ((s = c->cuda(cudaMemcpy(h.data(), sum.p, sum.bytes, cudaMemcpyDeviceToHost), "film copy")) != RX_OK) return s;
  for (size_t k = 0; k < h.size(); k++) film_rgb[k] = count(k / 3) > 0 ? h[k] / count(k / 3) : 0.0;
  if (film_sq) {
    if ((s = c->cuda(cudaMemcpy(h.data(), sq.p, sq.bytes, cudaMemcpyDeviceToHost), "film copy")) != RX_OK) return s;
    for (size_t k = 0; k < h.size(); k++) film_sq[k] = count(k / 3) > 0 ? h[k] / count(k / 3) : 0.0;
  }
  if (stats) *stats = st;
  return RX_OK;
}

rx_status rx_render_pt_batch(rx_context* c, const rx_batch_item* items, uint32_t n, rx_batch_options* opts,
                             rx_render_stats* stats) {
  if (!c) return RX_ERR_INVALID;
  if (!items || n == 0) return c->fail(RX_ERR_INVALID, "empty batch");
  if (n > 65535) return c->fail(RX_ERR_INVALID, "at most 65535 scenes per batch");
  std::vector<rx::PtJob> jobs(n);
  uint64_t pixels = 0;
  for (uint32_t k = 0; k < n; k++) {
    const rx_batch_item& it = items[k];
    if (!it.scene || !it.film_rgb) return c->fail(RX_ERR_INVALID, "batch item without scene or film");
    if (!it.scene->scene_ready) return c->fail(RX_ERR_STATE, "batch item scene not built");
    if (it.scene->device != c->device) return c->fail(RX_ERR_INVALID, "batch scenes must share the device");
    const rx_camera& cam = it.camera;
    if (cam.width == 0 || cam.height == 0 || cam.sight_dist == 0) return c->fail(RX_ERR_INVALID, "bad camera");
    if (it.options.spp == 0 || it.options.max_depth > 1000) return c->fail(RX_ERR_INVALID, "bad spp or max_depth");
    if (it.options.time_budget_s != 0.0f || it.options.reserved)
      return c->fail(RX_ERR_INVALID, "time_budget_s applies to rx_render_pt only; reserved 0");
    if (it.options.nee && it.scene->scene.num_lights == 0)
      return c->fail(RX_ERR_INVALID, "light sampling needs an emissive object");
    if (it.options.flags & ~RX_PT_GUIDED) return c->fail(RX_ERR_INVALID, "unknown flags");
    if (it.options.flags & RX_PT_GUIDED) {
      if (it.options.nee) return c->fail(RX_ERR_INVALID, "guiding applies to PathTracer (nee = 0)");
      if (!rx::guide_ready(it.scene->guide))
        return c->fail(RX_ERR_STATE, "guided batch item needs rx_guide_init on its scene's context");
    }
    jobs[k] = rx::PtJob{it.scene, cam, it.options, pixels};
    pixels += (uint64_t)cam.width * cam.height;
  }
  DeviceGuard g(c->device);
  DevBuf film;
  rx_status s;
  if ((s = c->cuda(film.alloc(pixels * 3 * sizeof(double)), "film")) != RX_OK) return s;
  cudaMemsetAsync(film.p, 0, film.bytes, c->stream);
  rx::PtRun run;
  run.paths_per_pass = opts ? opts->paths_per_pass : 0;
  run.use_graph = opts ? opts->use_graph != 0 : true;
  run.autotune = opts ? opts->autotune != 0 : false;
  rx::PtShape shape;
  rx_render_stats st{};
  if ((s = c->cuda(rx::render_pt_jobs(c, jobs.data(), (int)n, run, film.as<double>(), nullptr, &st, &shape, c->stream),
                   "render_pt_batch")) != RX_OK)
    return s;
  std::vector<double> h(pixels * 3);
  if ((s = c->cuda(cudaMemcpy(h.data(), film.p, film.bytes, cudaMemcpyDeviceToHost), "film copy")) != RX_OK) return s;
  for (uint32_t k = 0; k < n; k++) {
    size_t np = (size_t)items[k].camera.width * items[k].camera.height * 3;
    const double* src = h.data() + jobs[k].film_base * 3;
    for (size_t q = 0; q < np; q++) items[k].film_rgb[q] = src[q] / items[k].options.spp;
  }
  if (opts) {
    opts->chosen_blocks_per_sm = shape.blocks_per_sm;
    opts->chosen_stack = shape.stack;
    opts->chosen_paths_per_pass = shape.paths_per_pass;
  }
  if (stats) *stats = st;
  return RX_OK;
}

static rx_status render_bidirectional(rx_context* c, const rx_camera* cam, const rx_vcm_options* opts,
                                      double* film_rgb, rx_render_stats* stats) {
  if (!c) return RX_ERR_INVALID;
  if (!cam || !opts || !film_rgb) return c->fail(RX_ERR_INVALID, "null argument");
  if (!c->scene_ready) return c->fail(RX_ERR_STATE, "scene objects not built (rx_scene_set_objects, rx_build_accel)");
  if (cam->width == 0 || cam->height == 0 || cam->sight_dist == 0) return c->fail(RX_ERR_INVALID, "bad camera");
  if (opts->iterations == 0) return c->fail(RX_ERR_INVALID, "iterations must be positive");
  if (opts->max_depth > 21) return c->fail(RX_ERR_INVALID, "max_depth must be at most 21");
  if (!(opts->radius > 0.0f) || !(opts->alpha > 0.0f)) return c->fail(RX_ERR_INVALID, "radius and alpha must be positive");
  if (!(opts->time_budget_s >= 0.0f) || opts->reserved) return c->fail(RX_ERR_INVALID, "time_budget_s >= 0, reserved 0");
  if (c->scene.num_lights == 0) return c->fail(RX_ERR_INVALID, "vertex connection and merging needs an emitter");
  DeviceGuard g(c->device);
  size_t np = (size_t)cam->width * cam->height;
  DevBuf film;
  rx_status s;
  if ((s = c->cuda(film.alloc(np * 3 * sizeof(double)), "film")) != RX_OK) return s;
  cudaMemsetAsync(film.p, 0, film.bytes, c->stream);
  rx_render_stats st{};
  if ((s = c->cuda(rx::render_vcm(c, *cam, *opts, film.as<double>(), &st, c->stream), "render_vcm")) != RX_OK) return s;
  std::vector<double> h(np * 3);
  if ((s = c->cuda(cudaMemcpy(h.data(), film.p, film.bytes, cudaMemcpyDeviceToHost), "film copy")) != RX_OK) return s;
  const double iters = (double)(st.paths / np);  // iterations done (fewer under a time budget)
  for (size_t k = 0; k < h.size(); k++) film_rgb[k] = h[k] / iters;
  if (stats) *stats = st;
  return RX_OK;
}

rx_status rx_render_vcm(rx_context* c, const rx_camera* cam, const rx_vcm_options* opts, double* film_rgb,
                        rx_render_stats* stats) {
  if (!c) return RX_ERR_INVALID;
  if (opts && (opts->flags & ~RX_VCM_FULL_PATH_MIS)) return c->fail(RX_ERR_INVALID, "unknown VCM flags");
  return render_bidirectional(c, cam, opts, film_rgb, stats);
}

rx_status rx_render_bpt(rx_context* c, const rx_camera* cam, const rx_bpt_options* opts, double* film_rgb,
                        rx_render_stats* stats) {
  if (!c) return RX_ERR_INVALID;
  if (!opts) return c->fail(RX_ERR_INVALID, "null argument");
  if (opts->flags & ~RX_VCM_FULL_PATH_MIS) return c->fail(RX_ERR_INVALID, "unknown BPT flags");
  rx_vcm_options v{opts->iterations, opts->max_depth, 0u,        opts->flags | rx::kVcmBidirectional,
                   1.0f,             1.0f,            opts->seed, opts->time_budget_s,
                   0u};
  return render_bidirectional(c, cam, &v, film_rgb, stats);
}

rx_status rx_render_pm(rx_context* c, const rx_camera* cam, const rx_pm_options* opts, double* film_rgb,
                       rx_render_stats* stats) {
  if (!c) return RX_ERR_INVALID;
  if (!cam || !opts || !film_rgb) return c->fail(RX_ERR_INVALID, "null argument");
  if (!c->scene_ready) return c->fail(RX_ERR_STATE, "scene objects not built (rx_scene_set_objects, rx_build_accel)");
  if (cam->width == 0 || cam->height == 0 || cam->sight_dist == 0) return c->fail(RX_ERR_INVALID, "bad camera");
  if (opts->iterations == 0) return c->fail(RX_ERR_INVALID, "iterations must be positive");
  if (opts->max_depth > 21) return c->fail(RX_ERR_INVALID, "max_depth must be at most 21");
  if (!(opts->radius > 0.0f) || !(opts->alpha >= 0.0f) || opts->flags)
    return c->fail(RX_ERR_INVALID, "radius must be positive, alpha non-negative, flags 0");
  if (!(opts->time_budget_s >= 0.0f) || opts->reserved) return c->fail(RX_ERR_INVALID, "time_budget_s >= 0, reserved 0");
  if (c->scene.num_lights == 0) return c->fail(RX_ERR_INVALID, "photon mapping needs an emitter");
  DeviceGuard g(c->device);
  size_t np = (size_t)cam->width * cam->height;
  DevBuf film;
  rx_status s;
  if ((s = c->cuda(film.alloc(np * 3 * sizeof(double)), "film")) != RX_OK) return s;
  cudaMemsetAsync(film.p, 0, film.bytes, c->stream);
  rx_render_stats st{};
  if ((s = c->cuda(rx::render_pm(c, *cam, *opts, film.as<double>(), &st, c->stream), "render_pm")) != RX_OK) return s;
  std::vector<double> h(np * 3);
  if ((s = c->cuda(cudaMemcpy(h.data(), film.p, film.bytes, cudaMemcpyDeviceToHost), "film copy")) != RX_OK) return s;
  const double iters = (double)(st.paths / np);  // iterations done (fewer under a time budget)
  for (size_t k = 0; k < h.size(); k++) film_rgb[k] = h[k] / iters;
  if (stats) *stats = st;
  return RX_OK;
}

rx_status rx_accel_stats(rx_context* c, int64_t out[8]) {
  if (!c || !out) return RX_ERR_INVALID;
  if (!c->accel_ready) return c->fail(RX_ERR_STATE, "accelerator not built");
  std::memset(out, 0, 8 * sizeof(int64_t));
  out[0] = (int64_t)c->bvh.nodes.size();
  out[1] = c->bvh.max_depth;
  out[2] = (int64_t)c->ref.nodes.size();
  out[3] = c->ref.max_depth;
  out[4] = (int64_t)(c->tris.size() / 3);
  out[5] = (int64_t)c->ref.leaf_node.size();
  out[6] = c->bvh4.max_depth;
  out[7] = c->bvh8.max_depth;
  return RX_OK;
}

// Scratch of a closest-hit launch over n rays: n winner leaves + up to n queued rays.
static rx_status ensure_queue(rx_context* c, size_t n) {
  size_t need = rx::trace_scratch_bytes(std::max<size_t>(n, 1024));
  if (c->d_queue.bytes >= need) return RX_OK;
  return c->cuda(c->d_queue.alloc(need), "allocate closest-hit scratch");
}

rx_status rx_trace_closest_device(rx_context* c, const rx_ray* d_rays, uint32_t n, int32_t* d_tid, float* d_dist,
                                  void* stream) {
  if (!c) return RX_ERR_INVALID;
  if (!c->accel_ready) return c->fail(RX_ERR_STATE, "accelerator not built");
  if (n == 0) return RX_OK;
  if (!d_rays || !d_tid || !d_dist) return c->fail(RX_ERR_INVALID, "null buffer");
  if (reinterpret_cast<uintptr_t>(d_rays) % 16) return c->fail(RX_ERR_INVALID, "rays must be 16-byte aligned");
  DeviceGuard g(c->device);
  rx_status s = ensure_queue(c, n);
  if (s != RX_OK) return s;
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  const cudaEvent_t* ev = nullptr;
  if (c->timing_on && c->timing_used + 4 <= c->timing_ev.size()) {
    ev = &c->timing_ev[c->timing_used];
    c->timing_used += 4;
  }
  return c->cuda(rx::launch_trace_closest(c->accel, d_rays, n, d_tid, d_dist, c->d_queue.as<uint32_t>(),
                                          c->d_counters.as<unsigned long long>(), c->trace_cfg, st, ev),
                 "trace_closest launch");
}

rx_status rx_trace_set_timing(rx_context* c, int32_t max_calls) {
  if (!c || max_calls < 0 || max_calls > 4096) return c ? c->fail(RX_ERR_INVALID, "max_calls must be 0..4096") : RX_ERR_INVALID;
  DeviceGuard g(c->device);
  for (cudaEvent_t e : c->timing_ev) cudaEventDestroy(e);
  c->timing_ev.clear();
  c->timing_used = 0;
  c->timing_on = max_calls > 0;
  for (int32_t k = 0; k < 4 * max_calls; k++) {
    cudaEvent_t e;
    rx_status s = c->cuda(cudaEventCreate(&e), "create timing event");
    if (s != RX_OK) return s;
    c->timing_ev.push_back(e);
  }
  return RX_OK;
}

rx_status rx_trace_read_timing(rx_context* c, float* ms3, int32_t* calls) {
  if (!c || !calls) return RX_ERR_INVALID;
  DeviceGuard g(c->device);
  int32_t k = (int32_t)(c->timing_used / 4);
  if (ms3) {
    for (int32_t i = 0; i < k; i++) {
      const cudaEvent_t* e = &c->timing_ev[4 * (size_t)i];
      rx_status s = c->cuda(cudaEventSynchronize(e[3]), "timing events");
      if (s != RX_OK) return s;
      for (int j = 0; j < 3; j++) cudaEventElapsedTime(&ms3[3 * i + j], e[j], e[j + 1]);
    }
  }
  *calls = k;
  return RX_OK;
}

rx_status rx_trace_closest_reforder_device(rx_context* c, const rx_ray* d_rays, uint32_t n, int32_t* d_tid,
                                           float* d_dist, void* stream) {
  if (!c) return RX_ERR_INVALID;
  if (!c->accel_ready) return c->fail(RX_ERR_STATE, "accelerator not built");
  if (n == 0) return RX_OK;
  if (!d_rays || !d_tid || !d_dist) return c->fail(RX_ERR_INVALID, "null buffer");
  if (c->ref.max_depth >= 120) return c->fail(RX_ERR_UNSUPPORTED, "reference tree deeper than the walk stack");
  DeviceGuard g(c->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  return c->cuda(rx::launch_trace_reforder(c->accel, d_rays, n, d_tid, d_dist, c->d_counters.as<unsigned long long>(), st),
                 "trace_reforder launch");
}

rx_status rx_set_snapshots(rx_context* c, double every_s, rx_snapshot_fn fn, void* user) {
  if (!c) return RX_ERR_INVALID;
  if (!(every_s >= 0.0)) return c->fail(RX_ERR_INVALID, "every_s must be >= 0");
  c->snap_every = fn ? every_s : 0.0;
  c->snap_fn = every_s > 0 ? fn : nullptr;
  c->snap_user = user;
  return RX_OK;
}

rx_status rx_trace_set_binning(rx_context* c, int32_t cell_bits, int32_t dir_bits, int32_t dir_map) {
  if (!c) return RX_ERR_INVALID;
  const bool ok = cell_bits >= 3 && cell_bits <= 5 && dir_bits >= 1 &&
                  (dir_map == 0 ? dir_bits <= 3 && 3 * (cell_bits + dir_bits) <= 21
                                : dir_map == 1 && dir_bits <= 6 && 3 * cell_bits + 2 * dir_bits <= 21);
  if (!ok)
    return c->fail(RX_ERR_INVALID, "binning: cell_bits 3..5; dir_map 0: dir_bits 1..3, cell_bits + dir_bits <= 7; "
                                   "dir_map 1: dir_bits 1..6, 3 cell_bits + 2 dir_bits <= 21");
  c->trace_cfg.bin_cell_bits = cell_bits;
  c->trace_cfg.bin_dir_bits = dir_bits;
  c->trace_cfg.bin_dir_map = dir_map;
  return RX_OK;
}

rx_status rx_trace_set_staging(rx_context* c, uint32_t chunk_rays) {
  if (!c) return RX_ERR_INVALID;
  if (chunk_rays != 0 && chunk_rays < (1u << 16)) return c->fail(RX_ERR_INVALID, "chunk_rays: 0 or at least 65536");
  c->stage_rays = chunk_rays ? chunk_rays : (size_t)1 << 22;
  return RX_OK;
}

// Host buffers. The rays go to the device in chunks through a ring of three slots: the
// copies in on one stream, each slot's kernels (binning, walk, check, re-walk) on a
// stream of its own, the results back on a third, ordered per slot by events. The walk
// of a chunk holds every SM until its tail, when its blocks retire one by one; the next
// chunk's binning and walk, on the next slot's stream and already queued, take those SMs
// then, so the tail of one walk is filled by the start of the next (and the check of a
// chunk runs in the tail of the walk after it). A third slot keeps the copies in ahead
// of the kernels while a check waits for that tail. The chunks ramp up (a quarter, a
// half, then stage_rays: 2^22 by default, large enough for binning and the persistent
// walk) so that the first copy, the one no kernel hides, is short; on the 2^24-ray batch
// 10.50 ms a call at 2^22 against 10.59 at 2^23 and 10.85 at 2^21.
rx_status rx_trace_closest(rx_context* c, const rx_ray* rays, uint32_t n, int32_t* out_tid, float* out_dist) {
  if (!c) return RX_ERR_INVALID;
  if (!c->accel_ready) return c->fail(RX_ERR_STATE, "accelerator not built");
  if (n == 0) return RX_OK;
  if (!rays || !out_tid || !out_dist) return c->fail(RX_ERR_INVALID, "null buffer");
  DeviceGuard g(c->device);
  const size_t chunk = std::min<size_t>(n, c->stage_rays);
  std::vector<size_t> sizes;  // the chunk schedule
  for (size_t b = 0, sz = std::max<size_t>(chunk / 4, std::min<size_t>(chunk, (size_t)1 << 16)); b < n;) {
    const size_t m = std::min(sz, (size_t)n - b);
    sizes.push_back(m);
    b += m;
    sz = std::min(chunk, 2 * sz);
  }
  const int nring = (int)std::min<size_t>(rx_context::kRing, sizes.size());
  if (c->ring_chunk < chunk) {  // every slot is (re)made at the larger size when next used
    for (int k = 0; k < rx_context::kRing; k++)
      for (DevBuf* b : {&c->ring_rays[k], &c->ring_tid[k], &c->ring_dist[k], &c->ring_queue[k]}) b->release();
    c->ring_chunk = chunk;
  }
  for (int k = 0; k < nring; k++) {
    rx_status s;
    if (!c->ring_rays[k].p) {
      const size_t cap = c->ring_chunk;
      if ((s = c->cuda(c->ring_rays[k].alloc(cap * sizeof(rx_ray)), "staging")) != RX_OK) return s;
      if ((s = c->cuda(c->ring_tid[k].alloc(cap * 4), "staging")) != RX_OK) return s;
      if ((s = c->cuda(c->ring_dist[k].alloc(cap * 4), "staging")) != RX_OK) return s;
      if ((s = c->cuda(c->ring_queue[k].alloc(rx::trace_scratch_bytes(cap)), "staging")) != RX_OK) return s;
    }
    if (!c->ring_counters[k].p) {
      if ((s = c->cuda(c->ring_counters[k].alloc(8 * sizeof(unsigned long long)), "staging")) != RX_OK) return s;
      cudaMemset(c->ring_counters[k].p, 0, c->ring_counters[k].bytes);
    }
    if (!c->ring_stream[k] &&
        (s = c->cuda(cudaStreamCreateWithFlags(&c->ring_stream[k], cudaStreamNonBlocking), "staging streams")) != RX_OK)
      return s;
    for (cudaEvent_t& e : c->ring_ev[k])
      if (!e && (s = c->cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "staging events")) != RX_OK)
        return s;
  }
  cudaStream_t in = c->copy_stream[0], out = c->copy_stream[1];
  // the slots' streams start after whatever the context's stream holds, and the call
  // ends with all of them done
  cudaEvent_t start = c->ring_ev[0][2];
  cudaEventRecord(start, c->stream);
  cudaStreamWaitEvent(in, start, 0);
  size_t b = 0;
  for (size_t i = 0; i < sizes.size(); i++) {
    const int k = (int)(i % nring);
    const size_t m = sizes[i];
    cudaEvent_t* ev = c->ring_ev[k];  // [0] copied in, [1] traced, [2] copied out
    cudaStream_t run = c->ring_stream[k];
    if (i >= (size_t)nring) cudaStreamWaitEvent(in, ev[1], 0);  // the slot's previous rays are traced
    cudaMemcpyAsync(c->ring_rays[k].p, rays + b, m * sizeof(rx_ray), cudaMemcpyHostToDevice, in);
    cudaEventRecord(ev[0], in);
    cudaStreamWaitEvent(run, ev[0], 0);
    if (i >= (size_t)nring) cudaStreamWaitEvent(run, ev[2], 0);  // the slot's previous results are copied out
    cudaError_t e = rx::launch_trace_closest(c->accel, c->ring_rays[k].as<rx_ray>(), (uint32_t)m,
                                             c->ring_tid[k].as<int32_t>(), c->ring_dist[k].as<float>(),
                                             c->ring_queue[k].as<uint32_t>(),
                                             c->ring_counters[k].as<unsigned long long>(), c->trace_cfg, run);
    if (e != cudaSuccess) {
      cudaStreamSynchronize(in);
      for (int q = 0; q < nring; q++) cudaStreamSynchronize(c->ring_stream[q]);
      cudaStreamSynchronize(out);
      return c->cuda(e, "trace_closest launch");
    }
    cudaEventRecord(ev[1], run);
    cudaStreamWaitEvent(out, ev[1], 0);
    cudaMemcpyAsync(out_tid + b, c->ring_tid[k].p, m * 4, cudaMemcpyDeviceToHost, out);
    cudaMemcpyAsync(out_dist + b, c->ring_dist[k].p, m * 4, cudaMemcpyDeviceToHost, out);
    cudaEventRecord(ev[2], out);
    b += m;
  }
  rx_status r = c->cuda(cudaStreamSynchronize(in), "trace_closest");
  for (int q = 0; q < nring && r == RX_OK; q++) r = c->cuda(cudaStreamSynchronize(c->ring_stream[q]), "trace_closest");
  if (r == RX_OK) r = c->cuda(cudaStreamSynchronize(out), "trace_closest");
  return r;
}

rx_status rx_trace_set_config(rx_context* c, int32_t variant, int32_t blocks_per_sm) {
  if (!c) return RX_ERR_INVALID;
  if (variant < 0 || variant > 5 || blocks_per_sm < 1 || blocks_per_sm > 32)
    return c->fail(RX_ERR_INVALID, "variant must be 0..5 and blocks_per_sm 1..32");
  c->trace_cfg.variant = variant;
  c->trace_cfg.blocks_per_sm = blocks_per_sm;
  return RX_OK;
}

rx_status rx_trace_set_options(rx_context* c, int32_t check_mode, uint32_t bin_min, int32_t walk_stack) {
  if (!c) return RX_ERR_INVALID;
  if (check_mode != 0 && check_mode != 1) return c->fail(RX_ERR_INVALID, "check_mode must be 0 or 1");
  if (walk_stack != 0 && walk_stack != 32 && walk_stack != 64) return c->fail(RX_ERR_INVALID, "walk_stack: 0, 32 or 64");
  c->trace_cfg.check_thread = check_mode;
  c->trace_cfg.bin_min = bin_min;
  c->trace_cfg.walk_stack = walk_stack;
  return RX_OK;
}

rx_status rx_trace_counters(rx_context* c, uint64_t out[4], int reset) {
  if (!c || !out) return RX_ERR_INVALID;
  DeviceGuard g(c->device);
  unsigned long long h[4], r[rx_context::kRing][8];
  rx_status s = c->cuda(cudaDeviceSynchronize(), "counters");
  if (s != RX_OK) return s;
  cudaMemcpy(h, c->d_counters.p, sizeof h, cudaMemcpyDeviceToHost);
  for (int k = 0; k < 4; k++) out[k] = h[k];
  for (int k = 0; k < rx_context::kRing; k++)
    if (c->ring_counters[k].p) {
      cudaMemcpy(r[k], c->ring_counters[k].p, sizeof r[k], cudaMemcpyDeviceToHost);
      for (int j = 1; j < 4; j++) out[j] += r[k][j];
    }
  if (reset) {
    cudaMemset(c->d_counters.p, 0, c->d_counters.bytes);
    for (int k = 0; k < rx_context::kRing; k++)
      if (c->ring_counters[k].p) cudaMemset(c->ring_counters[k].p, 0, c->ring_counters[k].bytes);
  }
  return RX_OK;
}

}  // extern "C"
