// Reference VCM driver: loads a config through the reference's Renderer::loadConfig and
// runs VCMTracer::renderPixels (reference src/VCMTracer.cpp:6-143) once: a full
// progressive estimate of ITERS iterations starting from radius R0 with shrink exponent
// ALPHA, written as float64 RGB. The global random stream is first advanced by an
// amount set by RUN, so separate invocations are independent estimates (the golden
// script averages them and takes their spread as the standard error). One estimate per
// process: SceneObject::preprocessEmissionSampler appends to its area table without
// clearing it (SceneObject.cpp:107-116), so a second renderPixels in the same process
// would sample emitter triangles out of range.
//
// Test infrastructure only (builds where the reference sources are mounted).
//
//   vcm_driver <config.xml> <iters> <run> <r0> <alpha> <out_prefix> [threads]
#include "stdafx.h"
#include "Renderer.h"
#include "VCMTracer.h"

#include <chrono>
#include <cstdio>
#include <omp.h>
#include <string>
#include <vector>

class OracleVCM : public VCMTracer {
 public:
  explicit OracleVCM(Renderer* r) : VCMTracer(r) {}
  void set_iterations(unsigned n) { spp = n; }  // VCMTracer::spp is protected
};

int main(int argc, char** argv) {
  if (argc < 7) {
    fprintf(stderr, "usage: %s config.xml iters run r0 alpha out_prefix [threads]\n", argv[0]);
    return 2;
  }
  int iters = atoi(argv[2]), run = atoi(argv[3]);
  float r0 = (float)atof(argv[4]), alpha = (float)atof(argv[5]);
  std::string pre = argv[6];
  if (argc > 7) omp_set_num_threads(atoi(argv[7]));
  Renderer renderer;
  renderer.loadConfig(argv[1]);
  renderer.scene.buildObjKDTrees();  // Renderer::render, Renderer.cpp:47-51
  OracleVCM vcm(&renderer);
  vcm.setMaxDepth(renderer.mcRenderer ? renderer.mcRenderer->getMaxDepth() : 20);
  vcm.setRuntime(1e30);
  vcm.isDebug = true;
  vcm.alpha = alpha;
  vcm.set_iterations(iters);
  const Camera& cam = renderer.camera;
  size_t np = (size_t)cam.width * cam.height;
  std::vector<double> out(3 * np, 0.0);
  for (long k = 0; k < 1000003L * (run + 1); k++) RandGenerator::genFloat();
  auto t0 = std::chrono::steady_clock::now();
  vcm.setRadius(r0);
  std::vector<vec3f> img = vcm.renderPixels(cam);
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (size_t p = 0; p < np; p++)
    for (int c = 0; c < 3; c++) out[3 * p + c] = img[p][c];
  FILE* f = fopen((pre + ".img.f64").c_str(), "wb");
  fwrite(out.data(), 8, out.size(), f);
  fclose(f);
  printf("%d %d %d %d %.3f\n", cam.width, cam.height, iters, run, secs);
  return 0;
}
