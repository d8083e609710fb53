// Path-guiding network: sizes, parameter layout, the mixture of von Mises-Fisher lobes
// the network outputs, and the host-side state a context keeps for it.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "rx_pt.cuh"
#include "rx_wavefront.h"

namespace rx {
namespace guide {

constexpr int kIn = 80;        // encoded inputs (78 used + constant 1 + 0)
constexpr int kHid = 64;       // hidden width
constexpr int kOut = 64;       // output rows (40 used, rows 40..63 stay zero)
constexpr int kOutUsed = 40;   // 8 lobes x 5
constexpr int kLobes = 8;
constexpr int kFreq = 12;      // sin/cos frequencies per position coordinate
constexpr int kTile = 128;     // samples per CTA tile
constexpr int kRec = 16;       // floats per record: x, n, wo, wi, weight, 3 spare
constexpr int kLobeFloats = 6;  // per lobe: weight, kappa, mean xyz, weight x vMF normaliser
constexpr int kLobeStride = kLobes * kLobeFloats;  // floats per query

// Input width of layer l (0..4).
__host__ __device__ constexpr int layer_k(int l) { return l == 0 ? kIn : kHid; }
// FP32 parameters: layer l's [64][layer_k(l)] row-major block starts at layer_w(l).
__host__ __device__ constexpr int layer_w(int l) { return l == 0 ? 0 : 64 * kIn + (l - 1) * 64 * kHid; }
constexpr int kParams = 64 * kIn + 4 * 64 * kHid;  // 21504
// BF16 image: layer l's matrix in the shared-memory core-matrix layout at byte layer_img(l).
__host__ __device__ constexpr uint32_t layer_img(int l) { return (uint32_t)layer_w(l) * 2u; }
constexpr uint32_t kImgBytes = (uint32_t)kParams * 2u;  // 43008

// Axis-aligned box that normalises positions to [0, 1]^3 for the encoding.
struct Box {
  float mn[3], ext[3];
};

// pdf of direction w under a stored mixture (lobes of one query).
__device__ __forceinline__ float mix_pdf(const float* L, F3 w) {
  float q = 0.0f;
#pragma unroll
  for (int j = 0; j < kLobes; j++) {
    const float* l = L + j * kLobeFloats;
    float t = l[2] * w.x + l[3] * w.y + l[4] * w.z;
    q += l[5] * __expf(l[1] * (t - 1.0f));
  }
  return q;
}

// Samples a direction from the mixture: a lobe by weight (u0), then the vMF lobe about
// its mean (u1, u2) by inverting the cosine's distribution.
__device__ __forceinline__ F3 mix_sample(const float* L, float u0, float u1, float u2) {
  int j = 0;
  float acc = 0.0f;
  for (; j < kLobes - 1; j++) {
    acc += L[j * kLobeFloats];
    if (u0 < acc) break;
  }
  const float* l = L + j * kLobeFloats;
  float k = l[1];
  // cos = 1 + log(u + (1-u) e^{-2k}) / k
  float c = 1.0f + logf(u1 + (1.0f - u1) * __expf(-2.0f * k)) / k;
  c = fminf(fmaxf(c, -1.0f), 1.0f);
  float sn = sqrtf(fmaxf(0.0f, 1.0f - c * c));
  float sp, cp;
  sincospif(2.0f * u2, &sp, &cp);
  Frame f = frame_from(F3{l[2], l[3], l[4]});
  return to_world(f, F3{sn * cp, c, sn * sp});
}

}  // namespace guide

// Host-side state of a context's guiding network (rx_guide.cu).
struct GuideState;
void guide_free(GuideState* g);

// Launches the inference kernel over the `n` live paths of a wavefront: for each path
// whose hit is a guided surface, writes its mixture (guide::kLobeStride floats) to `lobes`.
cudaError_t guide_infer_paths(GuideState* g, const DevScene& S, const PathSoA& P, const unsigned* count,
                              const int2* hit, float* lobes, int grid, cudaStream_t s);
// `steps` Adam steps on the record buffer whose live count (at most n_max) is device-
// resident: step k trains on a window of `batch` records picked on the device, so no
// host synchronisation is needed.
cudaError_t guide_train_records(GuideState* g, const float* recs, const unsigned* count, uint32_t n_max,
                                int steps, cudaStream_t s);
bool guide_ready(const GuideState* g);
float guide_bsdf_fraction(const GuideState* g);
uint32_t guide_train_passes(const GuideState* g);
uint32_t guide_steps_per_pass(const GuideState* g);
uint32_t guide_warmup_passes(const GuideState* g);

}  // namespace rx
