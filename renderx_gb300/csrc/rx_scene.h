// Device scene for the light-transport kernels: per-object materials, per-triangle
// shading data and the emitter sampler, next to the closest-hit structures.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rx_device.h"

namespace rx {

enum MatKind : uint32_t {
  kDiffuse = 0,     // DiffuseMaterial (reference src/DiffuseMaterial.cpp)
  kGlossy = 1,      // GlossyMaterial, Phong lobe (src/GlossyMaterial.cpp)
  kRefractive = 2,  // RefractiveMaterial (src/RefractiveMaterial.cpp:132-269)
  kEmissive = 3,    // SceneEmissiveObject (src/SceneEmissiveObject.cpp)
  kPhong = 4,       // ScenePhongObject: glossy + diffuse (include/ScenePhongObject.h)
  kReflective = 5,  // SceneReflectiveObject: refractive with coeff -1
  kVPM = 6          // SceneVPMObject (src/SceneVPMObject.cpp)
};

struct DevObject {
  uint32_t material;
  uint32_t has_normals;
  uint32_t tri_begin, tri_count;
  float color[3];
  float coeff;
  float diffuse_color[3];
  float ior;
  float sigma_s[3], sigma_a[3];
  float g;
  float decay[3];
  float step_size;  // PhotonMap's ray-marching step in a medium
};

struct DevScene {
  DevAccel accel;
  const float4* slot_n;     // per BVH slot: 3 float4 shading normals; [0].w = object id bits
  const float4* tri_v;      // per triangle id: 3 float4 vertices
  const float4* tri_n;      // per triangle id: 3 float4 vertex normals (face normal when none)
  const uint32_t* tri_obj;  // per triangle id: object id
  const DevObject* objects;
  uint32_t num_objects;
  const float* light_cdf;   // cumulative area over emitter triangles (last = total)
  const uint32_t* light_tri;
  uint32_t num_lights;
  float light_area;         // total emitter area (Scene::SurfaceSampler totals)
};

}  // namespace rx
