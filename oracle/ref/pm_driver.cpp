// Reference PhotonMap driver: loads a config through the reference's Renderer::loadConfig
// and runs PhotonMap::renderPixels (reference src/Photonmap.cpp:12-138) once: the running
// mean of ITERS progressive iterations from base radius R0, written as float64 RGB. The
// global random stream is first advanced by an amount set by RUN, so separate invocations
// are independent estimates. One estimate per process (see vcm_driver.cpp).
//
// PhotonMap keeps its iteration count in a private member that nothing sets (it renders
// until killed), so this harness translation unit alone sees the class's members as
// public to set it; the reference's compiled code is unchanged (same layout).
//
// Test infrastructure only (builds where the reference sources are mounted).
//
//   pm_driver <config.xml> <iters> <run> <r0> <out_prefix> [threads]
#include "stdafx.h"
#include "Renderer.h"
#define private public
#include "Photonmap.h"
#undef private

#include <chrono>
#include <cstdio>
#include <omp.h>
#include <string>
#include <vector>

int main(int argc, char** argv) {
  if (argc < 6) {
    fprintf(stderr, "usage: %s config.xml iters run r0 out_prefix [threads]\n", argv[0]);
    return 2;
  }
  int iters = atoi(argv[2]), run = atoi(argv[3]);
  float r0 = (float)atof(argv[4]);
  std::string pre = argv[5];
  if (argc > 6) omp_set_num_threads(atoi(argv[6]));
  Renderer renderer;
  renderer.loadConfig(argv[1]);
  renderer.scene.buildObjKDTrees();  // Renderer::render, Renderer.cpp:47-51
  PhotonMap pm(&renderer);
  pm.setMaxDepth(renderer.mcRenderer ? renderer.mcRenderer->getMaxDepth() : 20);
  pm.setRuntime(1e30);
  pm.isDebug = true;
  pm.setRadius(r0);
  pm.spp = (unsigned)iters;
  const Camera& cam = renderer.camera;
  size_t np = (size_t)cam.width * cam.height;
  std::vector<double> out(3 * np, 0.0);
  for (long k = 0; k < 1000003L * (run + 1); k++) RandGenerator::genFloat();
  auto t0 = std::chrono::steady_clock::now();
  std::vector<vec3f> img = pm.renderPixels(cam);
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (size_t p = 0; p < np; p++)
    for (int c = 0; c < 3; c++) out[3 * p + c] = img[p][c];
  FILE* f = fopen((pre + ".img.f64").c_str(), "wb");
  fwrite(out.data(), 8, out.size(), f);
  fclose(f);
  printf("%d %d %d %d %.3f\n", cam.width, cam.height, iters, run, secs);
  return 0;
}
