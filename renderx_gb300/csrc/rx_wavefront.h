// Wavefront path state shared by the path tracer's stages and the guiding network's
// inference pass.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace rx {

// Path state, structure of arrays (one slot per live path).
struct PathSoA {
  float4* o;     // origin, w = sampling pdf of the current ray (MIS)
  float4* d;     // direction, w = unused
  float4* T;     // throughput, w = unused
  float4* L;     // accumulated radiance, w = unused
  int4* info;    // pixel, contact object, inside object, depth | last-specular << 8
  uint64_t* id;  // path id (random-number key)
};

}  // namespace rx
