// Drop-in GPU renderers behind the reference's renderer interface: MCRenderer subclasses
// (reference include/MCRenderer.h:145-148, the virtual renderPixels that
// Renderer::render calls, src/Renderer.cpp:47-51) whose renderPixels runs this
// library's path tracer, VCM, bidirectional path tracer or photon map through the C ABI
// (include/renderx.h). A program built against the reference swaps one in for the
// renderer ConfigManager created for the config's <Renderer><type>
// (src/ConfigManager.cpp:325-354): see make_gpu_renderer below.
//
// This header is compiled against the reference's own headers (it needs Renderer,
// Scene, Camera and MCRenderer); it is not part of the library build.
//
// The scene reaches the device from the reference's in-memory Scene: world-space
// vertices and triangles from Scene::tree (filled by Scene::buildKDTree,
// src/Scene.cpp:248-285, in object order with ObjSourceInformation), so the triangles
// the GPU traces are exactly those the reference's KDTree holds. The reference keeps
// material parameters in protected members, so the object table (material codes,
// colours, exponents, indices, media) and vertex normals come from the library's own
// reader of the same config file (rx_config_read); load() checks that the two agree
// on every object's triangle range and on every vertex, bit for bit.
#pragma once

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "MCRenderer.h"
#include "Renderer.h"
#include "renderx.h"

namespace rxa {

// The library context holding one reference Renderer's scene.
class GpuScene {
 public:
  GpuScene() = default;
  GpuScene(const GpuScene&) = delete;
  GpuScene& operator=(const GpuScene&) = delete;
  ~GpuScene() {
    if (ctx_) rx_destroy(ctx_);
    if (host_) rx_host_scene_free(host_);
  }

  // Reads the config's object table with the library's reader and compares it with the
  // reference's Scene (no device). Returns false with error() set on a mismatch.
  bool check(Renderer* r, const std::string& config_path) {
    if (!read(config_path)) return false;
    const KDTree& T = r->scene.tree;
    const float *v = nullptr, *vn = nullptr;
    const uint32_t *tv = nullptr, *to = nullptr, *tl = nullptr;
    const rx_object* objs = nullptr;
    uint32_t nv = 0, nt = 0, nobj = 0;
    rx_host_scene_arrays(host_, &v, &nv, &tv, &nt, &to, &tl, &vn, &objs, &nobj);
    if (nv != T.vertexPositionList.size() || nt != T.triangleList.size() || nobj != r->scene.objects.size())
      return fail("vertex, triangle or object counts differ from the reference's Scene");
    for (uint32_t i = 0; i < nv; i++) {
      const vec3f& p = T.vertexPositionList[i];
      if (std::memcmp(&p.x, v + 3 * (size_t)i, sizeof(float)) || std::memcmp(&p.y, v + 3 * (size_t)i + 1, 4) ||
          std::memcmp(&p.z, v + 3 * (size_t)i + 2, 4))
        return fail("world-space vertex " + std::to_string(i) + " differs from the reference's Scene");
    }
    for (uint32_t t = 0; t < nt; t++) {
      const KDTree::Triangle& tri = T.triangleList[t];
      const auto* osi = static_cast<const Scene::ObjSourceInformation*>(tri.sourceInformation);
      if (tri.vertexIndices.x != tv[3 * (size_t)t] || tri.vertexIndices.y != tv[3 * (size_t)t + 1] ||
          tri.vertexIndices.z != tv[3 * (size_t)t + 2] || osi->objID != to[t] || osi->triangleID != tl[t])
        return fail("triangle " + std::to_string(t) + " differs from the reference's Scene");
    }
    return true;
  }

  // check(), then a context on `device` with the reference's geometry, the library's
  // object table and normals, and the accelerator built.
  bool load(Renderer* r, const std::string& config_path, int device = 0) {
    if (!check(r, config_path)) return false;
    const float *v = nullptr, *vn = nullptr;
    const uint32_t *tv = nullptr, *to = nullptr, *tl = nullptr;
    const rx_object* objs = nullptr;
    uint32_t nv = 0, nt = 0, nobj = 0;
    rx_host_scene_arrays(host_, &v, &nv, &tv, &nt, &to, &tl, &vn, &objs, &nobj);
    if (rx_create(&ctx_, device) != RX_OK) return fail("no CUDA device for the GPU renderer");
    const KDTree& T = r->scene.tree;
    std::vector<uint32_t> idx(3 * (size_t)nt), obj(nt), loc(nt);
    for (uint32_t t = 0; t < nt; t++) {
      const KDTree::Triangle& tri = T.triangleList[t];
      const auto* osi = static_cast<const Scene::ObjSourceInformation*>(tri.sourceInformation);
      idx[3 * (size_t)t] = tri.vertexIndices.x;
      idx[3 * (size_t)t + 1] = tri.vertexIndices.y;
      idx[3 * (size_t)t + 2] = tri.vertexIndices.z;
      obj[t] = osi->objID;
      loc[t] = osi->triangleID;
    }
    rx_build_options bo = {0 /* the reference as GCC builds it */, 0, 0, 0};
    if (rx_scene_set_geometry(ctx_, &T.vertexPositionList[0].x, nv, idx.data(), nt, obj.data(), loc.data(), vn) !=
            RX_OK ||
        rx_scene_set_objects(ctx_, objs, nobj) != RX_OK || rx_build_accel(ctx_, &bo) != RX_OK)
      return fail(rx_last_error(ctx_));
    return true;
  }

  rx_context* ctx() const { return ctx_; }
  const rx_config_info& info() const { return info_; }
  const std::string& error() const { return err_; }
  bool fail(const std::string& m) {
    err_ = m;
    return false;
  }

 private:
  bool read(const std::string& config_path) {
    if (host_) return true;
    char e[512] = {0};
    if (rx_config_read(config_path.c_str(), &host_, &info_, e, sizeof e) != RX_OK) return fail(e);
    return true;
  }

  rx_context* ctx_ = nullptr;
  rx_host_scene* host_ = nullptr;
  rx_config_info info_{};
  std::string err_;
};

// The reference's Camera (include/Camera.h) as the ABI's camera.
inline rx_camera to_rx(const Camera& c) {
  rx_camera r{};
  r.width = (uint32_t)c.width;
  r.height = (uint32_t)c.height;
  r.sight_dist = c.sightDist;
  const vec3f* v[3] = {&c.position, &c.focus, &c.up};
  float* d[3] = {r.position, r.focus, r.up};
  for (int k = 0; k < 3; k++) {
    d[k][0] = v[k]->x;
    d[k][1] = v[k]->y;
    d[k][2] = v[k]->z;
  }
  return r;
}

// The FP64 film (rows from the top) as renderPixels' vector<vec3f>.
inline vector<vec3f> to_pixels(const std::vector<double>& film) {
  vector<vec3f> out(film.size() / 3);
  for (size_t p = 0; p < out.size(); p++)
    out[p] = vec3f((float)film[3 * p], (float)film[3 * p + 1], (float)film[3 * p + 2]);
  return out;
}

// Common part: the scene, the seed and the last call's status.
class GpuRenderer : public MCRenderer {
 public:
  GpuRenderer(Renderer* r, GpuScene* scene, uint64_t seed) : MCRenderer(r), scene_(scene), seed_(seed) {}
  rx_status status() const { return status_; }

 protected:
  // MCRenderer::runtime (the config's <time>) as the wall-time budget; 0 = none.
  float budget() const { return runtime > 0 && std::isfinite(runtime) && runtime < 1e9 ? (float)runtime : 0.0f; }
  GpuScene* scene_;
  uint64_t seed_;
  rx_status status_ = RX_OK;
};

// PathTracer (src/PathTracer.cpp:6-89) or PathTracerTest (src/PathTracerTest.cpp:7-86):
// samplesPerPixel samples per pixel (the cap when the config's <time> budget ends first).
class PathTracerGPU : public GpuRenderer {
 public:
  PathTracerGPU(Renderer* r, GpuScene* s, bool nee, uint64_t seed = 1) : GpuRenderer(r, s, seed), nee_(nee) {}
  vector<vec3f> renderPixels(const Camera& camera) override {
    rx_camera rc = to_rx(camera);
    rx_pt_options po = {(uint32_t)samplesPerPixel, maxDepth, 0, nee_ ? 1u : 0u, seed_, 0, 0, budget(), 0};
    std::vector<double> film(3 * (size_t)camera.width * camera.height);
    status_ = rx_render_pt(scene_->ctx(), &rc, &po, film.data(), nullptr, nullptr);
    return to_pixels(film);
  }

 private:
  bool nee_;
};

// VCMTracer (src/VCMTracer.cpp:6-143): samplesPerPixel iterations of width x height light
// paths from `radius` with shrink exponent `alpha` (VCMTracer::mergeRadius, alpha).
class VCMTracerGPU : public GpuRenderer {
 public:
  VCMTracerGPU(Renderer* r, GpuScene* s, float radius, float alpha, uint64_t seed = 1)
      : GpuRenderer(r, s, seed), radius_(radius), alpha_(alpha) {}
  vector<vec3f> renderPixels(const Camera& camera) override {
    rx_camera rc = to_rx(camera);
    rx_vcm_options vo = {(uint32_t)samplesPerPixel, maxDepth, 0, 0, radius_, alpha_, seed_, budget(), 0};
    std::vector<double> film(3 * (size_t)camera.width * camera.height);
    status_ = rx_render_vcm(scene_->ctx(), &rc, &vo, film.data(), nullptr);
    return to_pixels(film);
  }

 private:
  float radius_, alpha_;
};

// BidirectionalPathTracer (src/BidirectionalPathTracer.cpp:6-112).
class BidirectionalPathTracerGPU : public GpuRenderer {
 public:
  using GpuRenderer::GpuRenderer;
  vector<vec3f> renderPixels(const Camera& camera) override {
    rx_camera rc = to_rx(camera);
    rx_bpt_options bo = {(uint32_t)samplesPerPixel, maxDepth, 0, budget(), seed_};
    std::vector<double> film(3 * (size_t)camera.width * camera.height);
    status_ = rx_render_bpt(scene_->ctx(), &rc, &bo, film.data(), nullptr);
    return to_pixels(film);
  }
};

// PhotonMap (src/Photonmap.cpp:12-138): width x height photon paths per iteration.
class PhotonMapGPU : public GpuRenderer {
 public:
  PhotonMapGPU(Renderer* r, GpuScene* s, float radius, uint64_t seed = 1) : GpuRenderer(r, s, seed), radius_(radius) {}
  vector<vec3f> renderPixels(const Camera& camera) override {
    rx_camera rc = to_rx(camera);
    rx_pm_options po = {(uint32_t)samplesPerPixel, maxDepth, 0, 0, radius_, 0.0f, seed_, budget(), 0};
    std::vector<double> film(3 * (size_t)camera.width * camera.height);
    status_ = rx_render_pm(scene_->ctx(), &rc, &po, film.data(), nullptr);
    return to_pixels(film);
  }

 private:
  float radius_;
};

// The GPU renderer for the config's <Renderer><type> (as the library's reader classified
// it), with the config's maxDepth, spp (iterations) and <time> budget; null for a type
// without one. `alpha`: the VCM radius shrink exponent (the reference's default 2/3).
inline GpuRenderer* make_gpu_renderer(Renderer* r, GpuScene* s, float alpha = 0.6667f) {
  const rx_config_info& in = s->info();
  GpuRenderer* g = nullptr;
  switch (in.estimator) {
    case 0: g = new PathTracerGPU(r, s, false); break;
    case 1: g = new PathTracerGPU(r, s, true); break;
    case 2: g = new VCMTracerGPU(r, s, in.radius, alpha); break;
    case 3: g = new BidirectionalPathTracerGPU(r, s, 1); break;
    case 4: g = new PhotonMapGPU(r, s, in.radius); break;
    default: return nullptr;
  }
  g->setMaxDepth((int)in.max_depth);
  g->setSpp(in.spp ? (int)in.spp : 1);
  g->setRuntime(in.runtime_s > 0 ? in.runtime_s : 0.0);
  return g;
}

}  // namespace rxa
