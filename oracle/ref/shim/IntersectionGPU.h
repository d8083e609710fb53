/* Oracle build replacement for the reference's OpenGL intersection class
 * (include/IntersectionGPU.h): same static interface, no graphics stack. The oracle
 * always runs with <useGPU>0, where Scene never calls it (Scene.cpp:276). */
#pragma once
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "SimpleShape.h"
#include "macros.h"
#include "KDTree.h"

class IntersectionGPU {
 public:
  struct Ray {
    vec3f origin;
    vec3f direction;
    int last_tid;
    Ray() {}
    Ray(const vec3f& o, const vec3f& d) : origin(o), direction(d) {}
  };
  static std::vector<SimpleShape*> shapes;
  static std::vector<Ray> rayList;
  static void loadShapesToShader() { unavailable(); }
  static void loadKDTreeToShader(const KDTree&) { unavailable(); }
  static void init() { unavailable(); }
  static std::vector<vec4f> query(const std::vector<Ray>&) { unavailable(); return {}; }

 private:
  static void unavailable() {
    fprintf(stderr, "IntersectionGPU: the OpenGL path is not built in the oracle\n");
    abort();
  }
};
