// Reference hit driver: runs the reference's own KDTree (src/KDTree.cpp, compiled
// unmodified from the reference sources) on a scene and a ray batch read from raw
// files, and writes the closest-hit answers and the reference's own serialized tree.
//
// This is test infrastructure (the oracle), never product code. It exists only in
// the container that holds the reference sources; its outputs become the committed
// golden fixtures under tests/golden/.
//
// Usage: hit_driver <verts.f32> <tris.u32> <rays.f32> <out_prefix>
//   verts.f32 : nv*3 float32 world-space positions
//   tris.u32  : nt*3 uint32 vertex indices (object-major order, as Scene.cpp:248-285
//               concatenates them)
//   rays.f32  : n*6 float32 (origin xyz, direction xyz)
// Writes <out_prefix>.tid.i32 (n, -1 on miss), <out_prefix>.dist.f32 (n),
//        <out_prefix>.nodes.f32 (serializeForGPU node/min/max float4 arrays),
//        <out_prefix>.leaf.f32 (serializeForGPU leaf_v1 .w = triangle id order).
#include "stdafx.h"
#include "KDTree.h"
#include <cstdio>
#include <cstdlib>
#include <vector>

static std::vector<char> slurp(const char* path) {
  FILE* f = fopen(path, "rb");
  if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  std::vector<char> buf(n);
  if (n && fread(buf.data(), 1, n, f) != (size_t)n) { fprintf(stderr, "short read %s\n", path); exit(2); }
  fclose(f);
  return buf;
}

static void spit(const std::string& path, const void* data, size_t bytes) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(2); }
  if (bytes) fwrite(data, 1, bytes, f);
  fclose(f);
}

int main(int argc, char** argv) {
  if (argc != 5) { fprintf(stderr, "usage: %s verts tris rays out_prefix\n", argv[0]); return 2; }
  std::vector<char> vb = slurp(argv[1]), tb = slurp(argv[2]), rb = slurp(argv[3]);
  const float* v = (const float*)vb.data();
  const unsigned* t = (const unsigned*)tb.data();
  const float* r = (const float*)rb.data();
  size_t nv = vb.size() / 12, nt = tb.size() / 12, nr = rb.size() / 24;

  KDTree tree;
  for (size_t i = 0; i < nv; i++) tree.vertexPositionList.push_back(vec3f(v[3 * i], v[3 * i + 1], v[3 * i + 2]));
  for (size_t i = 0; i < nt; i++) {
    KDTree::Triangle tri;
    tri.vertexIndices = vec3ui(t[3 * i], t[3 * i + 1], t[3 * i + 2]);
    tri.sourceInformation = NULL;
    tree.triangleList.push_back(tri);
  }
  tree.build();  // default strategy BEST, KDTree.h:54

  std::vector<int> tid(nr);
  std::vector<float> dist(nr);
#pragma omp parallel for schedule(dynamic, 64)
  for (long i = 0; i < (long)nr; i++) {
    KDTree::Ray ray;
    ray.origin = vec3f(r[6 * i], r[6 * i + 1], r[6 * i + 2]);
    ray.direction = vec3f(r[6 * i + 3], r[6 * i + 4], r[6 * i + 5]);
    unsigned id = 0;
    float d = tree.intersect(ray, id, NULL);  // KDTree.h:50, public wrapper
    dist[i] = d;
    tid[i] = d >= 0 ? (int)id : -1;
  }
  std::string pre = argv[4];
  spit(pre + ".tid.i32", tid.data(), tid.size() * 4);
  spit(pre + ".dist.f32", dist.data(), dist.size() * 4);

  std::vector<vec4f> nodes, mins, maxs, l1, l2, l3;
  tree.serializeForGPU(nodes, mins, maxs, l1, l2, l3);
  std::vector<float> nf;
  for (size_t i = 0; i < nodes.size(); i++) {
    for (int k = 0; k < 4; k++) nf.push_back(nodes[i][k]);
    for (int k = 0; k < 4; k++) nf.push_back(mins[i][k]);
    for (int k = 0; k < 4; k++) nf.push_back(maxs[i][k]);
  }
  std::vector<float> lf;
  for (size_t i = 0; i < l1.size(); i++) lf.push_back(l1[i].w);
  spit(pre + ".nodes.f32", nf.data(), nf.size() * 4);
  spit(pre + ".leaf.f32", lf.data(), lf.size() * 4);
  // ray count, node count and leaf-triangle count for the caller's sanity check
  printf("%zu %zu %zu\n", nr, nodes.size(), l1.size());
  return 0;
}
