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

// One network as the kernels see it: its parameters, optimiser state and render
// schedule. A render of several scenes carries one network per guided scene; the
// grouped kernels take an array of these.
struct NetDev {
  const unsigned char* img;  // BF16 weight image (core-matrix layout)
  float *params, *m, *v, *grad;
  float* scratch;            // {sum of record weights, record count, loss} of the current step
  int* status;               // set when a bounded tensor-core wait gave up
  uint32_t* step;            // Adam steps taken
  guide::Box box;            // position-encoding box
  float lr;                  // Adam step size
  float frac;                // one-sample MIS: probability of sampling the BSDF
  uint32_t batch;            // records per Adam step
  uint32_t warmup;           // render passes before the first guided pass
  uint32_t train;            // render passes whose samples train the network
  uint32_t steps_per_pass;   // Adam steps after each training pass
};

// The records one network trains on: `cap` slots at `recs` (guide::kRec floats each),
// the live count at *count (device; null: all cap), `len` records per step.
struct RecSeg {
  const float* recs;
  const unsigned* count;
  uint32_t cap, len;
};

// Rows of a grouped inference: each network's rows are a segment padded to a multiple of
// kGroupRows (one inference CTA's four tiles), so a CTA's tiles share one network.
constexpr uint32_t kGroupRows = 4 * kTile;

}  // namespace guide

// Host-side state of a context's guiding network (rx_guide.cu).
struct GuideState;
void guide_free(GuideState* g);
bool guide_ready(const GuideState* g);
// The network's device view with its options (pointers into the state's buffers).
guide::NetDev guide_net(const GuideState* g);
// Sets the network kernels' shared-memory limits on the current device (call before
// capturing their launches in a graph).
void guide_prepare();

// Launches the inference kernel over a wavefront's live paths: for each path whose hit is
// a guided surface, writes its mixture (guide::kLobeStride floats) to `lobes`, else
// lobes[i * kLobeStride] = -1. scenes: the paths' scenes (index info.w >> 16).
// Ungrouped (rows null): one network (nets[0]) over queue entries 0..*count-1.
// Grouped: rows[r] = queue entry or -1 over segments seg[0..nnet] (multiples of
// kGroupRows), network k over rows [seg[k], seg[k + 1]). A network whose warm-up is not
// over at pass *pass (device) is skipped.
cudaError_t guide_infer_wave(const guide::NetDev* nets, int nnet, const DevScene* scenes, const PathSoA& P,
                             const unsigned* count, const int2* hit, float* lobes, const int* rows,
                             const uint32_t* seg, const uint32_t* pass, int sms, cudaStream_t s);
// Adam steps of every network on its own records: step k of a pass trains network j on
// the k-th window of its records (picked on the device); a network trains only while
// *pass < its train passes (pass null: always). Every launch size is fixed on the host, so
// the steps can be captured in a CUDA graph.
// batch_max: the largest `len` of the segments (sizes the launch).
cudaError_t guide_train_nets(const guide::NetDev* nets, const guide::RecSeg* segs, int nnet, int steps,
                             uint32_t batch_max, const uint32_t* pass, int sms, cudaStream_t s);

}  // namespace rx
