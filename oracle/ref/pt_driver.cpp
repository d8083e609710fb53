// Reference render driver: loads a config through the reference's own
// Renderer::loadConfig / ConfigManager::load and runs its path tracers for a fixed
// number of samples per pixel, writing per-pixel sums and sums of squares (float64) so
// golden images carry their own Monte Carlo standard error.
//
// Test infrastructure only (builds where the reference sources are mounted).
//
//   pt_driver <config.xml> <mode: pt|ptnee> <spp> <out_prefix> [threads]
//
// pt    : PathTracer's CPU estimator, PathTracer.cpp:26-68 (BSDF sampling only,
//         camera cosine + vignetting correction), restated around the protected
//         MCRenderer::samplePath because PathTracer's own spp is private and unbounded.
// ptnee : PathTracerTest's estimator, PathTracerTest.cpp:21-78, around the public
//         PathTracerTest::colorByConnectingLights.
#include "stdafx.h"
#include "Renderer.h"
#include "MCRenderer.h"
#include "PathTracerTest.h"
#include "SceneEmissiveObject.h"

#include <chrono>
#include <cstdio>
#include <omp.h>
#include <string>
#include <vector>

class OracleRun : public PathTracerTest {
 public:
  explicit OracleRun(Renderer* r) : PathTracerTest(r) {}

  // PathTracer.cpp:29-67 for one pixel sample; returns the sample value.
  vec3f sample_pt(const Camera& camera, int p, long& segments) {
    Path eyePath;
    Ray cameraRay = camera.generateRay(p);
    samplePath(eyePath, cameraRay, false);
    segments += (long)eyePath.size() - 1;
    if (!(eyePath.back().contactObject && eyePath.back().contactObject->emissive())) return vec3f(0, 0, 0);
    vec3f color(1, 1, 1);
    for (unsigned i = 0; i < eyePath.size(); i++) {
      color *= eyePath[i].color / eyePath[i].directionProb / eyePath[i].originProb;
      if (i != eyePath.size() - 1) {
        color *= eyePath[i].getCosineTerm();
        float dist = (eyePath[i + 1].origin - eyePath[i].origin).length();
        color *= eyePath[i].getRadianceDecay(dist);
      }
    }
    return renderer->camera.eliminateVignetting(color, p);
  }

  // PathTracerTest.cpp:23-78 for one pixel sample.
  vec3f sample_nee(const Camera& camera, int p, long& segments) {
    Path eyePath;
    Ray cameraRay = camera.generateRay(p);
    samplePath(eyePath, cameraRay, false);
    segments += (long)eyePath.size() - 1;
    vec3f throughput(1.f), color(0.f);
    bool lastSpecular = 1;
    float lastPdfW = 1.f;
    for (unsigned i = 1; i < eyePath.size(); i++) {
      if (eyePath[i].contactObject && eyePath[i].contactObject->emissive()) {
        vec3f contrib = ((SceneEmissiveObject*)(eyePath[i].contactObject))->getColor();
        float dirPdfA = eyePath[i].contactObject->getEmissionWeight() / eyePath[i].contactObject->totalArea;
        float mis = 1.f;
        if (i > 1 && !lastSpecular) {
          float cosine = eyePath[i].getContactNormal().dot(-eyePath[i - 1].direction);
          float dist = (eyePath[i].origin - eyePath[i - 1].origin).length();
          float dirPdfW = dirPdfA * dist * dist / std::abs(cosine);
          mis = lastPdfW / (lastPdfW + dirPdfW);
        }
        color += throughput * contrib * mis;
        break;
      }
      if (eyePath[i].directionSampleType == Ray::RANDOM) {
        segments++;  // shadow ray
        color += throughput * colorByConnectingLights(camera, eyePath[i], eyePath[i - 1]);
      }
      if (i + 1 >= eyePath.size() || eyePath[i].origin == eyePath[i + 1].origin) break;
      lastSpecular = (eyePath[i].directionSampleType == Ray::DEFINITE);
      lastPdfW = eyePath[i].directionProb;
      throughput *= eyePath[i].color * eyePath[i].getCosineTerm() / eyePath[i].directionProb;
      float dist = std::max((eyePath[i].origin - eyePath[i - 1].origin).length(), 1e-5f);
      throughput *= eyePath[i - 1].getRadianceDecay(dist);
    }
    return color;
  }
};

int main(int argc, char** argv) {
  if (argc < 5) {
    fprintf(stderr, "usage: %s config.xml pt|ptnee spp out_prefix [threads]\n", argv[0]);
    return 2;
  }
  std::string mode = argv[2];
  int spp = atoi(argv[3]);
  if (argc > 5) omp_set_num_threads(atoi(argv[5]));
  Renderer renderer;
  renderer.loadConfig(argv[1]);
  renderer.scene.buildObjKDTrees();  // Renderer::render, Renderer.cpp:47-51
  renderer.scene.preprocessEmissionSampler();
  OracleRun run(&renderer);
  run.setMaxDepth(renderer.mcRenderer ? renderer.mcRenderer->getMaxDepth() : 20);
  const Camera& cam = renderer.camera;
  int np = cam.width * cam.height;
  std::vector<double> sum(3 * (size_t)np, 0.0), sq(3 * (size_t)np, 0.0);
  long segments = 0;
  auto t0 = std::chrono::steady_clock::now();
  for (int s = 0; s < spp; s++) {
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : segments)
    for (int p = 0; p < np; p++) {
      vec3f c = mode == "pt" ? run.sample_pt(cam, p, segments) : run.sample_nee(cam, p, segments);
      for (int k = 0; k < 3; k++) {
        sum[3 * (size_t)p + k] += c[k];
        sq[3 * (size_t)p + k] += (double)c[k] * c[k];
      }
    }
  }
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::string pre = argv[4];
  FILE* f = fopen((pre + ".sum.f64").c_str(), "wb");
  fwrite(sum.data(), 8, sum.size(), f);
  fclose(f);
  f = fopen((pre + ".sq.f64").c_str(), "wb");
  fwrite(sq.data(), 8, sq.size(), f);
  fclose(f);
  printf("%d %d %d %ld %.3f\n", cam.width, cam.height, spp, segments, secs);
  return 0;
}
