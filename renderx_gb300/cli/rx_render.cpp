// rx_render: render a scene described by the reference's config file, as the reference's
// Renderer::loadConfig + MCRenderer::renderPixels + saveImagePFM do (reference
// src/Renderer.cpp:47-126, src/ConfigManager.cpp:166-405), through the C ABI.
//
//   rx_render config.xml [--out image.pfm] [--spp N] [--iterations N] [--light-paths N]
//             [--alpha A] [--seed S] [--guided] [--time SECONDS] [--snapshot-every SECONDS]
//             [--device D]
//
// The renderer type comes from the config (PathTracer / PT, PTtest, VCMTracer / VCM,
// BidirectionalPathTracer / BPT, PhotonMap / PM). As the reference, the render stops
// after the pass or iteration during which its time budget ran out (--time, else the
// config's <time> hours and minutes); the sample count (--spp, else <spp>, else 16 --
// 65,536 under a time budget; PT, PTtest and BPT) or iteration count (--iterations, else
// 8 -- 65,536 under a time budget; VCM and PM) caps it. Convergence snapshots go to
// <out stem>_time_<seconds>_iter_<s>.pfm every --snapshot-every seconds (default: the
// reference's 300 s timeStep under a time budget, else none; s = samples or iterations
// done - 1, the reference's loop index), the names MCRenderer::showCurrentResult writes
// (reference src/MCRenderer.cpp:465-490) and cmp/compare.cpp's calcRMSEs parses.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "renderx.h"

struct SnapshotFiles {
  std::string stem;
};

static void write_snapshot(void* user, double elapsed_s, double samples, const double* rgb, uint32_t w, uint32_t h) {
  const SnapshotFiles* f = static_cast<const SnapshotFiles*>(user);
  char name[1024];
  snprintf(name, sizeof name, "%s_time_%u_iter_%d.pfm", f->stem.c_str(), (unsigned)elapsed_s, (int)samples - 1);
  if (rx_write_pfm(name, w, h, rgb) == RX_OK) printf("snapshot %s\n", name);
}

static int fail(rx_context* c, const char* what) {
  fprintf(stderr, "rx_render: %s: %s\n", what, c ? rx_last_error(c) : "");
  if (c) rx_destroy(c);
  return 1;
}

int main(int argc, char** argv) {
  if (argc < 2 || !strcmp(argv[1], "-h") || !strcmp(argv[1], "--help")) {
    fprintf(stderr,
            "usage: %s config.xml [--out image.pfm] [--spp N] [--iterations N] [--light-paths N] [--alpha A]\n"
            "       [--seed S] [--guided] [--time SECONDS] [--snapshot-every SECONDS] [--device D]\n",
            argv[0]);
    return 2;
  }
  std::string cfg = argv[1], out;
  uint32_t spp = 0, iters = 0, light_paths = 0;
  double time_s = 0, snap_s = -1;
  float alpha = 0.6667f;
  uint64_t seed = 1;
  int device = 0;
  bool guided = false;
  for (int i = 2; i < argc; i++) {
    std::string a = argv[i];
    auto next = [&]() -> const char* { return i + 1 < argc ? argv[++i] : ""; };
    if (a == "--out") out = next();
    else if (a == "--spp") spp = (uint32_t)atoi(next());
    else if (a == "--iterations") iters = (uint32_t)atoi(next());
    else if (a == "--light-paths") light_paths = (uint32_t)atoi(next());
    else if (a == "--alpha") alpha = (float)atof(next());
    else if (a == "--seed") seed = strtoull(next(), nullptr, 10);
    else if (a == "--device") device = atoi(next());
    else if (a == "--guided") guided = true;
    else if (a == "--time") time_s = atof(next());
    else if (a == "--snapshot-every") snap_s = atof(next());
    else {
      fprintf(stderr, "rx_render: unknown option %s\n", a.c_str());
      return 2;
    }
  }
  rx_context* c = nullptr;
  if (rx_create(&c, device) != RX_OK) return fail(nullptr, "no CUDA device");
  rx_config_info info;
  auto t0 = std::chrono::steady_clock::now();
  if (rx_scene_load_config(c, cfg.c_str(), &info) != RX_OK) return fail(c, "loading the config");
  rx_build_options bo = {0, 4, 0, 0};
  if (rx_build_accel(c, &bo) != RX_OK) return fail(c, "building the accelerator");
  double load_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (out.empty()) out = info.save_path[0] ? info.save_path : "result.pfm";
  const uint32_t w = info.camera.width, h = info.camera.height;
  std::vector<double> film(3 * (size_t)w * h);
  rx_render_stats st{};
  if (time_s <= 0) time_s = info.runtime_s;
  const float budget = time_s > 0 ? (float)time_s : 0.0f;
  const uint32_t uncapped = 1u << 16;  // the cap under a time budget when none is given
  if (!spp) spp = info.spp ? info.spp : (budget > 0 ? uncapped : 16u);
  if (!iters) iters = budget > 0 ? uncapped : 8u;
  if (snap_s < 0) snap_s = budget > 0 ? 300.0 : 0.0;  // MCRenderer: timeStep = lastTime = 300
  SnapshotFiles snap_files{out.substr(0, out.rfind('.') == std::string::npos ? out.size() : out.rfind('.'))};
  if (snap_s > 0 && rx_set_snapshots(c, snap_s, write_snapshot, &snap_files) != RX_OK)
    return fail(c, "snapshots");
  if (info.estimator == 0 || info.estimator == 1) {
    rx_pt_options po = {spp, info.max_depth, 0, (uint32_t)info.estimator, seed, 0, 0, budget, 0};
    if (guided) {
      if (info.estimator != 0) return fail(c, "--guided applies to PathTracer");
      rx_guide_options go = {5e-3f, 0.5f, 1u << 18, 4, 16, 1, seed};
      if (rx_guide_init(c, &go, nullptr) != RX_OK) return fail(c, "guiding network");
      po.flags = RX_PT_GUIDED;
    }
    if (rx_render_pt(c, &info.camera, &po, film.data(), nullptr, &st) != RX_OK) return fail(c, "rendering");
    printf("%s: %u x %u, %.2f spp, depth %u: %.1f ms, %llu rays (load + build %.2f s)\n", info.renderer, w, h,
           (double)st.paths / ((double)w * h), po.max_depth, st.ms,
           (unsigned long long)(st.extension_rays + st.shadow_rays), load_s);
  } else if (info.estimator == 2) {
    float r = info.radius > 0 ? info.radius : 0.01f;
    rx_vcm_options vo = {iters, info.max_depth > 21 ? 21u : info.max_depth, light_paths, 0, r, alpha, seed, budget, 0};
    if (rx_render_vcm(c, &info.camera, &vo, film.data(), &st) != RX_OK) return fail(c, "rendering");
    printf("%s: %u x %u, %llu iterations, depth %u: %.1f ms, %llu rays (load + build %.2f s)\n", info.renderer, w,
           h, (unsigned long long)(st.paths / ((uint64_t)w * h)), vo.max_depth, st.ms,
           (unsigned long long)st.extension_rays, load_s);
  } else if (info.estimator == 3) {
    rx_bpt_options bo3 = {spp, info.max_depth > 21 ? 21u : info.max_depth, 0, budget, seed};
    if (rx_render_bpt(c, &info.camera, &bo3, film.data(), &st) != RX_OK) return fail(c, "rendering");
    printf("%s: %u x %u, %llu spp, depth %u: %.1f ms, %llu rays (load + build %.2f s)\n", info.renderer, w, h,
           (unsigned long long)(st.paths / ((uint64_t)w * h)), bo3.max_depth, st.ms,
           (unsigned long long)(st.extension_rays + st.shadow_rays), load_s);
  } else if (info.estimator == 4) {
    float r = info.radius > 0 ? info.radius : 0.01f;
    rx_pm_options pm = {iters, info.max_depth > 21 ? 21u : info.max_depth, light_paths, 0, r, 0.0f, seed, budget, 0};
    if (rx_render_pm(c, &info.camera, &pm, film.data(), &st) != RX_OK) return fail(c, "rendering");
    printf("%s: %u x %u, %llu iterations, depth %u: %.1f ms, %llu rays, %llu photons (load + build %.2f s)\n",
           info.renderer, w, h, (unsigned long long)(st.paths / ((uint64_t)w * h)), pm.max_depth, st.ms,
           (unsigned long long)st.extension_rays, (unsigned long long)st.merges, load_s);
  } else {
    fprintf(stderr, "rx_render: renderer type '%s' is not on this library's path\n", info.renderer);
    rx_destroy(c);
    return 3;
  }
  if (rx_write_pfm(out.c_str(), w, h, film.data()) != RX_OK) return fail(c, "writing the image");
  printf("wrote %s\n", out.c_str());
  rx_destroy(c);
  return 0;
}
