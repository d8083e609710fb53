// Reference BidirectionalPathTracer driver: loads a config through the reference's
// Renderer::loadConfig and runs BidirectionalPathTracer::renderPixels (reference
// src/BidirectionalPathTracer.cpp:6-112) once: the running mean of SPP iterations, each
// with one eye and one light subpath per pixel, written as float64 RGB. The global random
// stream is first advanced by an amount set by RUN, so separate invocations are
// independent estimates. One estimate per process, for the reason vcm_driver.cpp gives
// (the emission sampler's area table is appended to, never cleared).
//
// Test infrastructure only (builds where the reference sources are mounted).
//
//   bpt_driver <config.xml> <spp> <run> <out_prefix> [threads]
#include "stdafx.h"
#include "Renderer.h"
#include "BidirectionalPathTracer.h"

#include <chrono>
#include <cstdio>
#include <omp.h>
#include <string>
#include <vector>

class OracleBPT : public BidirectionalPathTracer {
 public:
  explicit OracleBPT(Renderer* r) : BidirectionalPathTracer(r) {}
  void set_spp(unsigned n) { spp = n; }  // BidirectionalPathTracer::spp is protected
};

int main(int argc, char** argv) {
  if (argc < 5) {
    fprintf(stderr, "usage: %s config.xml spp run out_prefix [threads]\n", argv[0]);
    return 2;
  }
  int spp = atoi(argv[2]), run = atoi(argv[3]);
  std::string pre = argv[4];
  if (argc > 5) omp_set_num_threads(atoi(argv[5]));
  Renderer renderer;
  renderer.loadConfig(argv[1]);
  renderer.scene.buildObjKDTrees();  // Renderer::render, Renderer.cpp:47-51
  OracleBPT bpt(&renderer);
  bpt.setMaxDepth(renderer.mcRenderer ? renderer.mcRenderer->getMaxDepth() : 20);
  bpt.setRuntime(1e30);
  bpt.isDebug = true;
  bpt.set_spp(spp);
  const Camera& cam = renderer.camera;
  size_t np = (size_t)cam.width * cam.height;
  std::vector<double> out(3 * np, 0.0);
  for (long k = 0; k < 1000003L * (run + 1); k++) RandGenerator::genFloat();
  auto t0 = std::chrono::steady_clock::now();
  std::vector<vec3f> img = bpt.renderPixels(cam);
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (size_t p = 0; p < np; p++)
    for (int c = 0; c < 3; c++) out[3 * p + c] = img[p][c];
  FILE* f = fopen((pre + ".img.f64").c_str(), "wb");
  fwrite(out.data(), 8, out.size(), f);
  fclose(f);
  printf("%d %d %d %d %.3f\n", cam.width, cam.height, spp, run, secs);
  return 0;
}
