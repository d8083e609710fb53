// Builds the reference-side adapter (renderx_gb300/adapters/reference_renderers.h)
// against the reference's own headers and objects, the way a program built from the
// reference would use it: the reference's Renderer loads a config (ConfigManager builds
// the Scene, its KDTree and the CPU renderer of the config's <type>), then a GPU renderer
// from the adapter replaces the CPU one and renders the config's camera.
//
// Test infrastructure (builds where the reference sources are mounted).
//
//   adapter_driver <config.xml> --check        compare the reference's Scene with the
//                                                library's reader of the config (no device)
//   adapter_driver <config.xml> <out.pfm>      render through the GPU renderer
//
// Exit codes: 0 ok, 1 mismatch or render error, 3 no CUDA device.
#include "stdafx.h"
#include "Renderer.h"

#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "adapters/reference_renderers.h"

static_assert(sizeof(vec3f) == 3 * sizeof(float), "vertex positions are packed float triples");

int main(int argc, char** argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s config.xml (--check | out.pfm)\n", argv[0]);
    return 2;
  }
  const std::string cfg = argv[1];
  Renderer renderer;
  renderer.loadConfig(cfg);  // ConfigManager::load: objects, camera, Scene::buildKDTree, the CPU renderer
  rxa::GpuScene scene;
  if (std::strcmp(argv[2], "--check") == 0) {
    if (!scene.check(&renderer, cfg)) {
      printf("check failed: %s\n", scene.error().c_str());
      return 1;
    }
    printf("check ok: %zu vertices, %zu triangles, %zu objects, renderer %s (estimator %d)\n",
           renderer.scene.tree.vertexPositionList.size(), renderer.scene.tree.triangleList.size(),
           renderer.scene.objects.size(), scene.info().renderer, scene.info().estimator);
    return 0;
  }
  if (!scene.load(&renderer, cfg)) {
    printf("load failed: %s\n", scene.error().c_str());
    return scene.ctx() ? 1 : 3;
  }
  std::unique_ptr<rxa::GpuRenderer> gpu(rxa::make_gpu_renderer(&renderer, &scene));
  if (!gpu) {
    printf("no GPU renderer for type %s\n", scene.info().renderer);
    return 1;
  }
  delete renderer.mcRenderer;  // the GPU renderer takes the CPU one's place
  renderer.mcRenderer = gpu.get();
  vector<vec3f> img = renderer.mcRenderer->renderPixels(renderer.camera);
  renderer.mcRenderer = nullptr;
  if (gpu->status() != RX_OK) {
    printf("render failed: %s\n", rx_last_error(scene.ctx()));
    return 1;
  }
  std::vector<double> rgb(3 * img.size());
  for (size_t p = 0; p < img.size(); p++)
    for (int c = 0; c < 3; c++) rgb[3 * p + c] = img[p][c];
  if (rx_write_pfm(argv[2], (uint32_t)renderer.camera.width, (uint32_t)renderer.camera.height, rgb.data()) != RX_OK) {
    printf("cannot write %s\n", argv[2]);
    return 1;
  }
  printf("rendered %dx%d to %s\n", renderer.camera.width, renderer.camera.height, argv[2]);
  return 0;
}
