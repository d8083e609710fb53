// Wavefront path tracing: the reference's PathTracer (BSDF sampling only,
// src/PathTracer.cpp:19-69) and PathTracerTest (next-event estimation with
// balance-heuristic MIS, src/PathTracerTest.cpp:7-136) estimators over the bounce loop
// of MCRenderer::samplePathIter (src/MCRenderer.cpp:151-267).
//
// Stages per bounce, each a grid-stride kernel whose work count lives in device memory
// (no host round trip inside a pass): extend (closest legal hit), shade (one scatter of
// the reference's bounce loop through rx_material.cuh, emission, next-event estimation
// with an inline shadow ray, Russian roulette) with queue compaction by warp ballot +
// one atomic per warp. Film accumulation is FP64.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "rx_bin.cuh"
#include "rx_guide.h"
#include "rx_internal.h"
#include "rx_material.cuh"
#include "rx_walk.cuh"
#include "rx_wavefront.h"

namespace rx {

struct PtParams {
  CamDev cam;
  uint64_t seed;
  uint32_t max_depth;
  uint32_t rr_mode;  // 0: reference RR at every bounce, 1: RR from depth 3 on
  uint32_t nee;      // 0: PathTracer, 1: PathTracerTest
  uint32_t pixels;
  uint32_t has_media;  // any medium object: camera rays look up their inside object
};

// One scene of a render: its geometry, estimator settings, and where its paths and film
// sit. A render of several scenes runs one wavefront over all their paths; a path
// carries its scene index (info.w >> 16).
struct SceneRec {
  DevScene S;
  PtParams P;
  uint64_t path_begin;  // concatenated passes: first global path index of the scene
  uint64_t pid_first;   // concatenated passes: the scene's first path id (0, or the paths
                        // that interleaved tuning passes took before)
  uint64_t film_base;   // first pixel of the scene in the shared film
  uint64_t paths;       // pixels x spp
  int32_t net;          // guiding network of the scene (index into the render's networks), -1: none
};

// Pass cursor in device memory, so that one captured pass replays unchanged. Two
// layouts of the paths over passes: concatenated (pass p takes global paths
// [p per_pass, (p + 1) per_pass) of the scenes' paths laid end to end) and interleaved
// (each pass takes the next quota[k] paths of every scene k, quota[k] proportional to
// the scene's paths, so every scene advances through its samples at the same pace and
// every pass holds the same mix: guided renders, whose networks warm up, train and
// guide on a schedule of passes, and autotuned ones, whose candidates are timed on
// consecutive passes). Interleaved passes keep each scene's cursor (paths taken) in
// device memory; the quotas can change between passes (the queue-size candidates).
struct PassState {
  uint64_t base, total;  // concatenated: first global path of the pass, all paths
  uint32_t per_pass, npaths;
  uint32_t pass;         // passes done (the guiding schedule reads it)
  uint32_t interleaved;
};

// Interleaved layout: per scene, the paths taken so far and the quota of each pass.
struct Layout {
  uint32_t* off;        // the current pass's offset of each scene's paths (nr + 1)
  uint64_t* taken;      // paths of each scene taken by earlier passes
  const uint32_t* quota;  // paths of each scene per pass
};

// A path's id: its index within its scene (the random-number key) and, in the top 24
// bits, its slot in the pass's generation order (training records refer to it).
constexpr int kLocalShift = 40;
constexpr uint64_t kPidMask = (1ull << kLocalShift) - 1;

__device__ __forceinline__ int scene_of(const SceneRec* R, int nr, uint64_t g) {
  int lo = 0, hi = nr - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (R[mid].path_begin <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// -------------------------------------------------------------------------------------
// Camera (reference src/Camera.cpp:4-47, 78-96)
// -------------------------------------------------------------------------------------
__device__ __forceinline__ F3 camera_dir(const CamDev& c, float xp, float yp) {
  float x = xp - c.width * 0.5f, y = c.height * 0.5f - yp;
  return normalize(c.front * c.sight + c.right * x + c.up * y);
}

// Interleaved passes: the share of scene k in the current pass.
__host__ __device__ __forceinline__ uint32_t pass_share(uint64_t paths, uint64_t taken, uint32_t quota) {
  if (taken >= paths) return 0u;
  const uint64_t left = paths - taken;
  return left < quota ? (uint32_t)left : quota;
}

// Interleaved passes: offsets off[0..nr] of each scene's paths in the generation order
// of the current pass (one block).
__global__ void __launch_bounds__(256) k_layout(const SceneRec* R, int nr, Layout L) {
  __shared__ uint32_t part[256];
  const int per = (nr + 255) / 256, k0 = threadIdx.x * per, k1 = min(nr, k0 + per);
  uint32_t sum = 0;
  for (int k = k0; k < k1; k++) sum += pass_share(R[k].paths, L.taken[k], L.quota[k]);
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {  // inclusive scan of the per-thread sums
    uint32_t v = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t acc = part[threadIdx.x] - sum;
  for (int k = k0; k < k1; k++) {
    L.off[k] = acc;
    acc += pass_share(R[k].paths, L.taken[k], L.quota[k]);
  }
  if (threadIdx.x == 255) L.off[nr] = part[255];
}

// End of an interleaved pass: each scene's cursor moves past its share (one block).
__global__ void k_layout_advance(int nr, Layout L) {
  for (int k = threadIdx.x; k < nr; k += blockDim.x) L.taken[k] += L.off[k + 1] - L.off[k];
}

// Scene k with off[k] <= i < off[k + 1].
__device__ __forceinline__ int scene_at(const uint32_t* off, int nr, uint32_t i) {
  int lo = 0, hi = nr - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void k_generate(const SceneRec* R, int nr, PassState* ps, Layout L, PathSoA S, unsigned* count) {
  uint32_t np;
  const bool inter = ps->interleaved != 0;
  if (inter) {
    np = L.off[nr];
  } else {
    const uint64_t left = ps->base < ps->total ? ps->total - ps->base : 0;
    np = (uint32_t)(left < ps->per_pass ? left : ps->per_pass);
  }
  const uint64_t base = ps->base;
  uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < np; i += stride) {
    int sc;
    uint64_t pid;  // path index within its scene (random-number key)
    if (inter) {
      sc = scene_at(L.off, nr, i);
      pid = L.taken[sc] + (i - L.off[sc]);
    } else {
      uint64_t g = base + i;
      sc = scene_of(R, nr, g);
      pid = R[sc].pid_first + (g - R[sc].path_begin);
    }
    const PtParams& P = R[sc].P;
    uint32_t pixel = (uint32_t)(pid % P.pixels);
    int x = pixel % P.cam.width, y = pixel / P.cam.width;
    Rng rng(P.seed, pid, 0);
    float jx = rng.next(), jy = rng.next();
    F3 d = camera_dir(P.cam, x + jx, y + jy);
    float w = 1.0f;
    if (!P.nee) {
      // camera ray's cosine term (Camera::getWorldNormal = front, Ray::getCosineTerm)
      // over the pixel-centre cosine of eliminateVignetting
      F3 dc = camera_dir(P.cam, x + 0.5f, y + 0.5f);
      w = fmaxf(fabsf(dot(P.cam.front, d)), 1e-6f) / fabsf(dot(dc, P.cam.front));
    }
    int inside = P.has_media ? find_inside(R[sc].S, P.cam.pos, d, kNone) : kNone;
    S.o[i] = make_float4(P.cam.pos.x, P.cam.pos.y, P.cam.pos.z, 1.0f);
    S.d[i] = make_float4(d.x, d.y, d.z, 0.0f);
    S.T[i] = make_float4(w, w, w, 0.0f);
    S.L[i] = make_float4(0, 0, 0, 0);
    S.info[i] = make_int4((int)pixel, kCameraObj, inside, (sc << 16) | (1 << 8));
    S.id[i] = pid | ((uint64_t)i << kLocalShift);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *count = np;
    ps->npaths = np;
  }
}

// The extension rays' lanes for walk_persistent (kWalk4P): path `order[r]` (binned
// order) or r of the queue, its scene's 4-wide BVH, the closest legal hit
// (NoSelfIntersectionCondition through leaf_test, as trace_cond4); the answer to hit[].
struct ExtendLane {
  const SceneRec* R;
  PathSoA S;
  uint32_t n;
  const uint32_t* __restrict__ order;
  int2* hit;
  const DevScene* sc = nullptr;
  uint32_t i = 0;
  int contact = kNone, inside = kNone;
  bool cond = false;
  PHit best{-1, INFINITY};

  __device__ bool begin(uint32_t r, F3& o, F3& d) {
    if (r >= n) return false;
    i = order ? __ldg(&order[r]) : r;
    const float4 o4 = S.o[i], d4 = S.d[i];
    const int4 inf = S.info[i];
    const bool camera = (inf.w & 255) == 0;  // the camera ray's first query has no condition
    sc = &R[(uint32_t)inf.w >> 16].S;
    contact = camera ? kNone : inf.y;
    inside = camera ? kNone : inf.z;
    cond = !(contact == kNone && inside == kNone);
    best = PHit{-1, INFINITY};
    o = f3(o4);
    d = f3(d4);
    return true;
  }
  __device__ const float4* nodes() const { return sc->accel.bvh4; }
  __device__ float limit() const { return best.t; }
  __device__ void leaf(int first, int count, F3 o, F3 d) {
    leaf_test<false>(*sc, first, count, o, d, cond, contact, inside, best);
  }
  __device__ void end() { hit[i] = make_int2(best.tid, __float_as_int(best.t)); }
};

// Closest legal hit of each live path's ray on persistent warps (kWalk4P): the same
// answers as k_extend<kWalk4S>, with lanes refilled from `cursor` (zero at launch)
// instead of each thread walking its share of the queue to the end.
__global__ void __launch_bounds__(128, 8) k_extend_p(const SceneRec* R, PathSoA S, const unsigned* count,
                                                     const uint32_t* __restrict__ order, int2* hit,
                                                     unsigned long long* rays, unsigned long long* cursor) {
  const uint32_t n = *count;
  ExtendLane L{R, S, n, order, hit};
  walk_persistent<4, kShortStack, 64>(L, cursor);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(rays, (unsigned long long)n);
}
// Bin keys of the live paths' next rays (counting sort input; rx_bin.cuh).
__global__ void k_path_keys(const SceneRec* R, PathSoA S, const unsigned* count, uint32_t* keys, uint32_t* hist) {
  uint32_t n = *count;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const DevAccel& A = R[(uint32_t)S.info[i].w >> 16].S.accel;
    uint32_t k = ray_key(A.lo, A.hi, S.o[i], S.d[i]);
    keys[i] = k;
    atomicAdd(&hist[k], 1u);
  }
}

// Closest legal hit of each live path's ray; `order` (optional) visits the paths in
// binned order.
template <int STACK>
__global__ void __launch_bounds__(128) k_extend(const SceneRec* R, PathSoA S, const unsigned* count,
                                                const uint32_t* __restrict__ order, int2* hit,
                                                unsigned long long* rays) {
  uint32_t n = *count;
  uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
    uint32_t i = order ? __ldg(&order[j]) : j;
    float4 o = S.o[i], d = S.d[i];
    int4 inf = S.info[i];
    bool camera = (inf.w & 255) == 0;  // the camera ray's first query has no condition
    const DevScene& SC = R[(uint32_t)inf.w >> 16].S;
    PHit h = trace_walk<false, STACK>(SC, f3(o), f3(d), INFINITY, camera ? kNone : inf.y, camera ? kNone : inf.z);
    hit[i] = make_int2(h.tid, __float_as_int(h.t));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(rays, (unsigned long long)n);
}

__device__ __forceinline__ void film_add(double* sum, double* sq, int pixel, F3 L) {
  double* s = sum + 3 * (size_t)pixel;
  atomicAdd(s, (double)L.x);
  atomicAdd(s + 1, (double)L.y);
  atomicAdd(s + 2, (double)L.z);
  if (sq) {
    double* q = sq + 3 * (size_t)pixel;
    atomicAdd(q, (double)L.x * L.x);
    atomicAdd(q + 1, (double)L.y * L.y);
    atomicAdd(q + 2, (double)L.z * L.z);
  }
}

// PathTracerTest::colorByConnectingLights (src/PathTracerTest.cpp:88-136) at vertex `v`
// (the ray leaving it), reached by `in`: a light point by area, two-sided emission,
// balance-heuristic weight against the BSDF's sampling pdf.
template <int STACK>
__device__ F3 connect_light(const DevScene& SC, const CamDev& cam, const PV& in, const PV& v, Rng& rng,
                            unsigned& shadows) {
  float ru = rng.next() * SC.light_area;
  int lo = 0, hi = (int)SC.num_lights - 1;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (__ldg(&SC.light_cdf[mid]) < ru) lo = mid + 1;
    else hi = mid;
  }
  int lt = (int)__ldg(&SC.light_tri[lo]);
  TriGeom lg = tri_geom(SC, lt);
  float u1 = rng.next(), u2 = rng.next();
  float su1 = sqrtf(u1);
  float bu = 1.0f - su1, bv = u2 * su1;
  F3 xl = lg.v0 * bu + lg.v1 * bv + lg.v2 * (1.0f - bu - bv);
  F3 ld = v.o - xl;
  float dist = length(ld);
  ld = ld * (1.0f / dist);
  PV out = v;
  out.d = -ld;
  F3 f = bsdf_of(SC, cam, in, out);
  if (lum(f) < 1e-7f) return {0, 0, 0};
  F3 nl = world_normal(lg, SC.objects[lg.obj].has_normals, xl);
  float cos_l = fminf(fabsf(dot(nl, ld)), 1.0f);
  if (cos_l < 1e-6f) return {0, 0, 0};
  float cos_s = 1.0f;
  if (v.contact != kNone) cos_s = fminf(fabsf(dot(contact_normal(SC, cam, v), out.d)), 1.0f);
  float bpdf = dir_pdf(SC, cam, in, out, false);
  shadows++;
  PHit sh = trace_walk<true, STACK>(SC, v.o, out.d, dist - 1e-5f, v.contact, v.inside);  // testVisibility
  if (sh.tid >= 0) return {0, 0, 0};
  float pdfa = 1.0f / SC.light_area;
  float pdfw = pdfa * dist * dist / cos_l;
  float mis = pdfw / (pdfw + bpdf);
  return f3v(SC.objects[lg.obj].color) * f * (cos_l * cos_s / (pdfa * dist * dist) * mis);
}

// Guided sampling state of a wavefront (all null / zero when guiding is off). A scene's
// network (SceneRec::net) guides from pass nets[net].warmup on and takes training
// records while the pass is below nets[net].train.
struct GuideIO {
  const guide::NetDev* nets;
  float* lobes;        // per live path: guide::kLobeStride floats, lobes[0] < 0 = not guided
  float* recs;         // training records (guide::kRec floats) or null
  unsigned* rec_count;
  uint32_t rec_cap;
  float4* lpath;       // radiance of each pass-local path at its end (training) or null
};

// The diffuse / glossy / Phong scatter of the eye path with its direction drawn by
// one-sample MIS: from the material's own lobe with probability `frac`, else from the
// guiding mixture G; the sampling density is the mixture of both. Russian roulette,
// the Phong lobe choice and the BSDF values are the plain scatter's, so the estimator's
// expectation is unchanged.
static __device__ PV scatter_guided(const DevScene& S, const PV& in, Hit3 h, bool russian, Rng& rng, const float* G,
                                    float frac) {
  const DevObject& ob = S.objects[h.obj];
  F3 x = in.o + in.d * h.dist;
  PV o = pv_term(x);
  o.pixel = in.pixel;
  o.contact = h.obj;
  o.ctri = h.tri;
  o.inside = in.inside;
  TriGeom g = tri_geom(S, h.tri);
  F3 n = world_normal(g, S.objects[g.obj].has_normals, x);
  uint32_t kind = ob.material;
  if (kind == kPhong) kind = rng.next() < 0.5f ? kGlossy : kDiffuse;
  bool from_bsdf = rng.next() < frac;
  float u0 = rng.next(), u1 = rng.next(), u2 = rng.next();
  o.flags = kDirRandom;
  if (kind == kDiffuse) {
    F3 c = ob.material == kPhong ? f3v(ob.diffuse_color) : f3v(ob.color);
    if (dot(in.d, n) > 0.0f) {  // leaving: pass through (not guided)
      o.d = in.d;
      o.c = {1, 1, 1};
      o.dprob = 1.0f;
      o.flags = 0;
      return o;
    }
    F3 w = from_bsdf ? to_world(frame_from(n), hemi_cos(1.0f, u1, u2)) : guide::mix_sample(G, u0, u1, u2);
    float p = maxc(c);
    if (russian && rng.next() >= p) {
      o.dprob = 1.0f - p;
      return o;  // d = 0, c = 0: the path ends
    }
    float pdf = frac * cos_lobe_pdf(n, w, 1.0f) + (1.0f - frac) * guide::mix_pdf(G, w);
    // no contribution below the surface; at its rim (cosine under the clamp of
    // Ray::getCosineTerm) the path ends as in the plain diffuse scatter
    bool front = dot(n, in.d) <= 0.0f && dot(n, w) >= kCosMin;
    if (!front || !(pdf > 0.0f)) return o;  // end
    o.d = w;
    o.c = c * (1.0f / RX_PI);
    o.dprob = (russian ? p : 1.0f) * pdf;
    return o;
  }
  F3 c = f3v(ob.color);
  F3 r = n * (-dot(n, in.d) * 2.0f) + in.d;
  F3 w = from_bsdf ? to_world(frame_from(r), hemi_cos(ob.coeff, u1, u2)) : guide::mix_sample(G, u0, u1, u2);
  F3 val = {0, 0, 0};
  if (dot(n, in.d) <= 0.0f && dot(n, w) >= 0.0f) {
    float rw = dot(r, w);
    if (rw > 0.0f) val = c * powf(rw, ob.coeff);
  }
  float pdf = frac * cos_lobe_pdf(r, w, ob.coeff) + (1.0f - frac) * guide::mix_pdf(G, w);
  if ((val.x == 0.0f && val.y == 0.0f && val.z == 0.0f) || !(pdf > 0.0f)) return o;
  o.d = w;
  o.c = val;
  o.dprob = pdf;
  if (russian) {
    float p = maxc(c);
    if (rng.next() < p) {
      o.dprob *= p;
    } else {
      o.d = {0, 0, 0};
      o.c = {0, 0, 0};
      o.dprob = 1.0f - p;
    }
  }
  return o;
}

// One bounce of MCRenderer::samplePathIter plus the estimator's bookkeeping.
template <int STACK>
__global__ void __launch_bounds__(128) k_shade(const SceneRec* R, const PassState* ps, PathSoA S,
                                               const unsigned* count, const int2* hit, PathSoA N, unsigned* next_count,
                                               double* film_sum, double* film_sq, unsigned long long* shadow_rays,
                                               GuideIO G) {
  uint32_t n = *count;
  uint32_t stride = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  unsigned shadows = 0;
  // every lane of a warp walks the same number of iterations (ballots need all 32)
  uint32_t nwarp_iter = (n + stride - 1) / stride;
  for (uint32_t it = 0; it < nwarp_iter; it++) {
    uint32_t i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
    bool cont = false;
    PV nx;
    F3 T{}, L{}, Tb{};
    int4 inf{};
    uint64_t pid = 0;
    int depth = 0;
    bool rec = false;  // a guided vertex whose path continues: a training record
    uint32_t sc = 0;
    uint32_t local = 0;  // the path's slot in the pass's generation order
    if (i < n) {
      float4 o4 = S.o[i], d4 = S.d[i], T4 = S.T[i], L4 = S.L[i];
      inf = S.info[i];
      pid = S.id[i];
      local = (uint32_t)(pid >> kLocalShift);
      depth = inf.w & 255;
      bool last_spec = (inf.w >> 8) & 1;
      sc = (uint32_t)inf.w >> 16;
      const DevScene& SC = R[sc].S;
      const PtParams& P = R[sc].P;
      T = f3(T4);
      L = f3(L4);
      PV cur = pv_term(f3(o4));
      cur.d = f3(d4);
      cur.contact = inf.y;
      cur.inside = inf.z;
      cur.pixel = inf.x;
      cur.flags = (depth == 0 || !last_spec) ? kDirRandom : 0u;  // the camera ray is RANDOM
      int2 h = hit[i];
      Rng rng(P.seed, pid & kPidMask, 16u + 32u * (uint32_t)depth);
      const int net = G.nets ? R[sc].net : -1;
      const bool training = net >= 0 && G.recs && ps->pass < G.nets[net].train;
      bool done = true;
      if (h.x >= 0) {  // a ray that hits nothing ends the path (samplePathIter's termRay)
        Hit3 hh{(int)__ldg(&SC.tri_obj[h.x]), h.x, __int_as_float(h.y)};
        bool russian = P.rr_mode == 0 || depth >= 3;
        bool guided = net >= 0 && G.lobes && !P.nee && ps->pass >= G.nets[net].warmup &&
                      __ldg(&G.lobes[(size_t)i * guide::kLobeStride]) >= 0.0f;
        if (guided) {
          nx = scatter_guided(SC, cur, hh, russian, rng, G.lobes + (size_t)i * guide::kLobeStride,
                              G.nets[net].frac);
          leak_kill(SC, P.cam, cur, nx);
        } else {
          nx = scatter_step(SC, P.cam, cur, hh, false, russian, rng);
        }
        float dist = length(nx.o - cur.o);
        bool killed = length(nx.d) < 0.5f;
        bool capped = !killed && depth + 1 > (int)P.max_depth;
        if (!P.nee) {
          // PathTracer.cpp:48-60: colour/directionProb/originProb of every ray, cosine
          // and transmittance of every ray but the last
          T = T * decay_of(SC, cur.inside, dist);
          Tb = T;
          T = T * (nx.c * (1.0f / (nx.dprob * nx.oprob)));
          if (killed && is_emissive(SC, nx.contact)) L = L + T;
          if (!killed && !capped) {
            T = T * cos_term(SC, P.cam, nx);
            done = false;
            // a training sample: a sampled direction at a diffuse / glossy / Phong
            // surface seen from outside any object
            uint32_t m = SC.objects[hh.obj].material;
            rec = training && cur.inside == kNone && (nx.flags & kDirRandom) && nx.contact == hh.obj &&
                  (m == kDiffuse || m == kGlossy || m == kPhong);
          }
        } else if (is_emissive(SC, nx.contact)) {
          // PathTracerTest.cpp:37-56: two-sided emission, MIS against light sampling
          float mis = 1.0f;
          if (depth > 0 && !last_spec) {
            float cosine = dot(contact_normal(SC, P.cam, nx), -cur.d);
            float pdfw = (1.0f / SC.light_area) * dist * dist / fabsf(cosine);
            mis = o4.w / (o4.w + pdfw);
          }
          L = L + T * f3v(SC.objects[nx.contact].color) * mis;
        } else if (!capped) {
          if ((nx.flags & kDirRandom) && SC.num_lights > 0) L = L + T * connect_light<STACK>(SC, P.cam, cur, nx, rng, shadows);
          if (!killed) {
            T = T * (nx.c * (cos_term(SC, P.cam, nx) / nx.dprob));
            T = T * decay_of(SC, cur.inside, fmaxf(dist, 1e-5f));
            done = false;
          }
        }
      }
      if (done) {
        // a sample that is not finite is dropped: it comes from a direction the 24-bit
        // generator draws with probability density zero (a cosine lobe's pole at
        // u = 0), where the reference's arithmetic divides by zero; one such sample
        // would poison a pixel's FP64 sum at very high sample counts
        const bool finite = isfinite(L.x) && isfinite(L.y) && isfinite(L.z);
        if (finite && (L.x != 0.0f || L.y != 0.0f || L.z != 0.0f))
          film_add(film_sum, film_sq, (int)(R[sc].film_base + (uint32_t)inf.x), L);
        if (training && G.lpath) G.lpath[local] = make_float4(L.x, L.y, L.z, 0.0f);
      } else {
        cont = true;
      }
    }
    // training record: position, shading normal, outgoing and incident directions,
    // throughput before this vertex, pass-local path index (weights follow the pass)
    unsigned rm = __ballot_sync(0xffffffffu, rec);
    if (rm) {
      unsigned rb = 0;
      int leader = __ffs(rm) - 1;
      if (lane == leader) rb = atomicAdd(G.rec_count, (unsigned)__popc(rm));
      rb = __shfl_sync(0xffffffffu, rb, leader);
      uint32_t j = rb + __popc(rm & ((1u << lane) - 1));
      if (rec && j < G.rec_cap) {
        F3 ns = contact_normal(R[sc].S, R[sc].P.cam, nx);
        float4* r = reinterpret_cast<float4*>(G.recs + (size_t)j * guide::kRec);
        float4 d4 = S.d[i];
        r[0] = make_float4(nx.o.x, nx.o.y, nx.o.z, ns.x);
        r[1] = make_float4(ns.y, ns.z, -d4.x, -d4.y);
        r[2] = make_float4(-d4.z, nx.d.x, nx.d.y, nx.d.z);
        r[3] = make_float4(Tb.x, Tb.y, Tb.z, __uint_as_float(local));
      }
    }
    // compaction: warp ballot, one atomic per warp
    unsigned m = __ballot_sync(0xffffffffu, cont);
    if (m) {
      unsigned base = 0;
      int leader = __ffs(m) - 1;
      if (lane == leader) base = atomicAdd(next_count, (unsigned)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (cont) {
        uint32_t j = base + __popc(m & ((1u << lane) - 1));
        N.o[j] = make_float4(nx.o.x, nx.o.y, nx.o.z, nx.dprob);
        N.d[j] = make_float4(nx.d.x, nx.d.y, nx.d.z, 0.0f);
        N.T[j] = make_float4(T.x, T.y, T.z, 0.0f);
        N.L[j] = make_float4(L.x, L.y, L.z, 0.0f);
        N.info[j] = make_int4(inf.x, nx.contact, nx.inside,
                              (int)(sc << 16) | (depth + 1) | (((nx.flags & kDirRandom) ? 0 : 1) << 8));
        N.id[j] = pid;
      }
    }
  }
  for (int s2 = 16; s2 > 0; s2 >>= 1) shadows += __shfl_xor_sync(0xffffffffu, shadows, s2);
  if (lane == 0 && shadows) atomicAdd(shadow_rays, (unsigned long long)shadows);
}

// The next queue's length, and the extension walk's refill cursor for the next bounce
// (kWalk4P: every k_extend_p launch of a pass is followed by this one, so the cursor is
// zero when the next starts).
__global__ void k_zero(unsigned* p, unsigned long long* cursor) {
  *p = 0;
  *cursor = 0ull;
}
__global__ void k_advance(PassState* ps) {
  ps->base += ps->per_pass;
  ps->pass += 1;
}

// Whether any network takes training records in this pass.
__device__ __forceinline__ bool any_training(const guide::NetDev* nets, int nnet, uint32_t pass) {
  for (int j = 0; j < nnet; j++)
    if (pass < nets[j].train) return true;
  return false;
}

// Start of a pass: clears the raw record count and every network's record count.
__global__ void k_records_begin(const guide::NetDev* nets, int nnet, const PassState* ps, unsigned* raw_count,
                                unsigned* net_count) {
  const uint32_t pass = ps->pass;
  for (int j = threadIdx.x; j < nnet; j += blockDim.x)
    if (pass < nets[j].train) net_count[j] = 0;
  if (threadIdx.x == 0) *raw_count = 0;
}

// Training samples of a finished pass: each record's weight is the luminance of its
// path's final radiance over the throughput before the vertex, i.e. (BSDF x cosine x
// incident radiance) / (sampling density) at the vertex. Records with a positive weight
// go to their network's region of `out` (x, n, wo, wi, weight, 0, 0, 0): network j's
// records at [rbase[j], rbase[j] + rcap[j]), counted in net_count[j] (which may pass
// rcap[j]: the surplus is dropped). A record's scene is the scene of its path's slot in
// the pass (off: the interleaved layout's offsets).
__global__ void k_record_weights(const SceneRec* R, int nr, const uint32_t* off, const PassState* ps,
                                 const guide::NetDev* nets, int nnet, const float* recs, const unsigned* count,
                                 uint32_t cap, const float4* lpath, float* out, unsigned* net_count,
                                 const uint32_t* rbase, const uint32_t* rcap) {
  const uint32_t pass = ps->pass;
  if (!any_training(nets, nnet, pass)) return;
  uint32_t n = min(*count, cap);
  const int lane = threadIdx.x & 31;
  uint32_t stride = gridDim.x * blockDim.x;
  uint32_t iters = (n + stride - 1) / stride;
  for (uint32_t it = 0; it < iters; it++) {
    uint32_t i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
    float4 a{}, b{}, c{}, d{};
    float w = 0.0f;
    int net = -1;
    if (i < n) {
      const float4* r = reinterpret_cast<const float4*>(recs + (size_t)i * guide::kRec);
      a = r[0];
      b = r[1];
      c = r[2];
      d = r[3];
      const uint32_t local = __float_as_uint(d.w);
      net = R[scene_at(off, nr, local)].net;
      float4 L = lpath[local];
      F3 q{d.x > 0.0f ? L.x / d.x : 0.0f, d.y > 0.0f ? L.y / d.y : 0.0f, d.z > 0.0f ? L.z / d.z : 0.0f};
      w = lum(q);
      if (!(w < 1e30f)) w = 0.0f;
      if (net < 0 || pass >= nets[net].train) w = 0.0f;
    }
    const bool keep = w > 0.0f;
    // lanes that keep a record of the same network share one atomic
    const unsigned peers = __match_any_sync(0xffffffffu, keep ? net : -1);
    if (keep) {
      const int leader = __ffs(peers) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(&net_count[net], (unsigned)__popc(peers));
      base = __shfl_sync(peers, base, leader);
      const uint32_t j = base + __popc(peers & ((1u << lane) - 1));
      if (j < rcap[net]) {
        float4* o = reinterpret_cast<float4*>(out + (size_t)(rbase[net] + j) * guide::kRec);
        o[0] = a;
        o[1] = b;
        o[2] = c;
        o[3] = make_float4(w, 0.0f, 0.0f, 0.0f);
      }
    }
  }
}

// Grouped inference input: the live paths of scenes whose network guides in this pass,
// sorted by network into segments padded to guide::kGroupRows rows (a counting sort:
// count, scan, scatter, pad). ncount / cursor: one counter per network.
__device__ __forceinline__ int active_net(const SceneRec* R, const guide::NetDev* nets, const int4& inf,
                                          uint32_t pass) {
  const int net = R[(uint32_t)inf.w >> 16].net;
  return net >= 0 && pass >= nets[net].warmup ? net : -1;
}
__global__ void k_net_count(const SceneRec* R, const guide::NetDev* nets, const PassState* ps, PathSoA S,
                            const unsigned* count, unsigned* ncount) {
  const uint32_t n = *count, pass = ps->pass;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t iters = (n + stride - 1) / stride;
  const int lane = threadIdx.x & 31;
  for (uint32_t it = 0; it < iters; it++) {
    const uint32_t i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
    const int net = i < n ? active_net(R, nets, S.info[i], pass) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, net);
    if (net >= 0 && lane == __ffs(peers) - 1) atomicAdd(&ncount[net], (unsigned)__popc(peers));
  }
}
// One block: seg[j] = padded offsets of the networks' segments; clears the counters
// the scatter uses.
__global__ void __launch_bounds__(256) k_net_scan(int nnet, const unsigned* ncount, uint32_t* seg,
                                                  unsigned* cursor) {
  __shared__ uint32_t part[256];
  const int per = (nnet + 255) / 256, k0 = threadIdx.x * per, k1 = min(nnet, k0 + per);
  auto padded = [](unsigned c) { return (c + guide::kGroupRows - 1) / guide::kGroupRows * guide::kGroupRows; };
  uint32_t sum = 0;
  for (int k = k0; k < k1; k++) sum += padded(ncount[k]);
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int o = 1; o < 256; o <<= 1) {
    uint32_t v = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t acc = part[threadIdx.x] - sum;
  for (int k = k0; k < k1; k++) {
    seg[k] = acc;
    cursor[k] = 0;
    acc += padded(ncount[k]);
  }
  if (threadIdx.x == 255) seg[nnet] = part[255];
}
__global__ void k_net_scatter(const SceneRec* R, const guide::NetDev* nets, const PassState* ps, PathSoA S,
                              const unsigned* count, const uint32_t* seg, unsigned* cursor, int* rows) {
  const uint32_t n = *count, pass = ps->pass;
  const uint32_t stride = gridDim.x * blockDim.x;
  const uint32_t iters = (n + stride - 1) / stride;
  const int lane = threadIdx.x & 31;
  for (uint32_t it = 0; it < iters; it++) {
    const uint32_t i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
    const int net = i < n ? active_net(R, nets, S.info[i], pass) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, net);
    if (net >= 0) {
      const int leader = __ffs(peers) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(&cursor[net], (unsigned)__popc(peers));
      base = __shfl_sync(peers, base, leader);
      rows[seg[net] + base + __popc(peers & ((1u << lane) - 1))] = (int)i;
    }
  }
}
// Padding rows of each segment (after its ncount[j] live rows) are -1; then the count is
// cleared for the next sort (block j owns network j).
__global__ void k_net_pad(int nnet, unsigned* ncount, const uint32_t* seg, int* rows) {
  const int j = blockIdx.x;
  if (j >= nnet) return;
  for (uint32_t r = seg[j] + ncount[j] + threadIdx.x; r < seg[j + 1]; r += blockDim.x) rows[r] = -1;
  __syncthreads();
  if (threadIdx.x == 0) ncount[j] = 0;
}

// -------------------------------------------------------------------------------------
// Host driver
// -------------------------------------------------------------------------------------
static cudaError_t alloc_soa(PathSoA& s, std::vector<DevBuf>& bufs, size_t n) {
  size_t sizes[6] = {16, 16, 16, 16, 16, 8};
  void** ptrs[6] = {(void**)&s.o, (void**)&s.d, (void**)&s.T, (void**)&s.L, (void**)&s.info, (void**)&s.id};
  for (int k = 0; k < 6; k++) {
    bufs.emplace_back();
    cudaError_t e = bufs.back().alloc(sizes[k] * n);
    if (e != cudaSuccess) return e;
    *ptrs[k] = bufs.back().p;
  }
  return cudaSuccess;
}

PtParams make_pt_params(const rx_context* c, const rx_camera& cam, const rx_pt_options& opt) {
  PtParams P{};
  auto v3 = [](const float* p) { return F3{p[0], p[1], p[2]}; };
  auto hn = [](F3 a) {
    float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return l > 0 ? F3{a.x / l, a.y / l, a.z / l} : a;
  };
  auto hc = [](F3 l, F3 r) { return F3{l.y * r.z - l.z * r.y, l.z * r.x - l.x * r.z, l.x * r.y - l.y * r.x}; };
  F3 pos = v3(cam.position), foc = v3(cam.focus), up = v3(cam.up);
  P.cam.pos = pos;
  P.cam.front = hn(F3{foc.x - pos.x, foc.y - pos.y, foc.z - pos.z});
  P.cam.right = hn(hc(P.cam.front, up));
  P.cam.up = hc(P.cam.right, P.cam.front);
  P.cam.sight = (float)cam.sight_dist;
  P.cam.width = (int)cam.width;
  P.cam.height = (int)cam.height;
  P.seed = opt.seed;
  P.max_depth = opt.max_depth;
  P.rr_mode = opt.rr_mode;
  P.nee = opt.nee;
  P.pixels = cam.width * cam.height;
  for (const rx_object& o : c->objects) P.has_media |= o.material == RX_MAT_VPM;
  return P;
}

namespace {

// W.ctr slot of the persistent extension walk's refill cursor (slots 0 and 1 count rays,
// 8 onwards hold the unsigned queue counts).
constexpr int kExtendCursor = 40;

// Device buffers of one wavefront render.
struct Wave {
  const SceneRec* R;
  int nr;
  PassState* ps;
  PathSoA A, B;
  int2* hit;
  unsigned long long* ctr;  // [0] extension rays, [1] shadow rays
  unsigned* cnt;            // [0], [1] queue lengths, [2] raw training records
  double *film, *sq;
  uint32_t loops;           // bounce stages per pass (max depth cap + 1)
  uint32_t *keys, *order, *hist;  // ray binning of bounce rays (null: off)
  Layout L;                 // interleaved passes (L.off null: concatenated)
  int sms;
  // guiding (nets null: off)
  const guide::NetDev* nets;
  int nnet;
  const DevScene* scenes;   // the scenes' geometry, for the inference kernel
  float* lobes;             // mixture per live path
  float* recs;              // raw training records (null: no network trains)
  uint32_t rec_cap;
  float4* lpath;            // each pass slot's final radiance
  float* train;             // records by network (weights computed)
  unsigned* net_count;      // per network: records in its region
  const uint32_t *rbase, *rcap;
  const guide::RecSeg* segs;
  int steps;                // Adam steps per training pass (the most any network takes)
  uint32_t batch_max;
  unsigned *ncount, *cursor;  // grouped inference sort (nnet > 1)
  uint32_t* seg;
  int* rows;
};

// Bins the queue's rays (bounces after the camera rays) and returns the visiting order.
const uint32_t* enqueue_binning(const Wave& W, PathSoA cur, const unsigned* cc, int grid, cudaStream_t s) {
  if (!W.order) return nullptr;
  cudaMemsetAsync(W.hist, 0, kRayBins * sizeof(uint32_t), s);
  k_path_keys<<<grid, 256, 0, s>>>(W.R, cur, cc, W.keys, W.hist);
  scan_bins(W.hist, W.hist + kRayBins, s);
  k_ray_scatter<<<grid, 256, 0, s>>>(W.keys, 0, cc, W.hist, W.order);
  return W.order;
}

// The guiding mixtures of the live paths whose scene's network guides in this pass: one
// network over the queue, or several over the queue sorted by network.
cudaError_t enqueue_infer(const Wave& W, const PathSoA& cur, const unsigned* cc, int grid, cudaStream_t s) {
  const uint32_t* pass = &W.ps->pass;
  if (W.nr == 1)  // one scene, one network: the queue as it is
    return guide_infer_wave(W.nets, 1, W.scenes, cur, cc, W.hit, W.lobes, nullptr, nullptr, pass, W.sms, s);
  k_net_count<<<grid, 256, 0, s>>>(W.R, W.nets, W.ps, cur, cc, W.ncount);
  k_net_scan<<<1, 256, 0, s>>>(W.nnet, W.ncount, W.seg, W.cursor);
  k_net_scatter<<<grid, 256, 0, s>>>(W.R, W.nets, W.ps, cur, cc, W.seg, W.cursor, W.rows);
  k_net_pad<<<W.nnet, 128, 0, s>>>(W.nnet, W.ncount, W.seg, W.rows);
  return guide_infer_wave(W.nets, W.nnet, W.scenes, cur, cc, W.hit, W.lobes, W.rows, W.seg, pass, W.sms, s);
}

// One pass: (layout), generate, `loops` x (extend, guiding inference, clear the next
// queue, shade), (training), advance the cursor. Everything is a kernel on `s` with
// device-resident counts and schedule, so the pass can be captured into a CUDA graph
// once and replayed.
template <int STACK>
cudaError_t enqueue_pass(const Wave& W, int grid, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  if (W.L.off) k_layout<<<1, 256, 0, s>>>(W.R, W.nr, W.L);
  if (W.recs) k_records_begin<<<1, 256, 0, s>>>(W.nets, W.nnet, W.ps, W.cnt + 2, W.net_count);
  k_generate<<<grid, 256, 0, s>>>(W.R, W.nr, W.ps, W.L, W.A, W.cnt);
  const GuideIO G{W.nets, W.lobes, W.recs, W.cnt + 2, W.rec_cap, W.lpath};
  PathSoA cur = W.A, nxt = W.B;
  unsigned *cc = W.cnt, *cn = W.cnt + 1;
  for (uint32_t d = 0; d < W.loops; d++) {
    const uint32_t* order = d > 0 ? enqueue_binning(W, cur, cc, grid, s) : nullptr;
    if constexpr (STACK == kWalk4P)  // persistent: the blocks that stay resident (8 per SM)
      k_extend_p<<<W.sms * 8, 128, 0, s>>>(W.R, cur, cc, order, W.hit, W.ctr, W.ctr + kExtendCursor);
    else
      k_extend<STACK><<<grid, 128, 0, s>>>(W.R, cur, cc, order, W.hit, W.ctr);
    if (W.nets && e == cudaSuccess) e = enqueue_infer(W, cur, cc, grid, s);
    k_zero<<<1, 1, 0, s>>>(cn, W.ctr + kExtendCursor);
    k_shade<STACK><<<grid, 128, 0, s>>>(W.R, W.ps, cur, cc, W.hit, nxt, cn, W.film, W.sq, W.ctr + 1, G);
    std::swap(cur, nxt);
    std::swap(cc, cn);
  }
  if (W.recs) {
    k_record_weights<<<grid, 128, 0, s>>>(W.R, W.nr, W.L.off, W.ps, W.nets, W.nnet, W.recs, W.cnt + 2, W.rec_cap,
                                          W.lpath, W.train, W.net_count, W.rbase, W.rcap);
    if (e == cudaSuccess) e = guide_train_nets(W.nets, W.segs, W.nnet, W.steps, W.batch_max, &W.ps->pass, W.sms, s);
  }
  if (W.L.off) k_layout_advance<<<1, 256, 0, s>>>(W.nr, W.L);
  k_advance<<<1, 1, 0, s>>>(W.ps);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t enqueue_pass_shape(const Wave& W, const PtShape& sh, int sms, cudaStream_t s) {
  int grid = sms * sh.blocks_per_sm;
  if (sh.stack == kWalk4P) return enqueue_pass<kWalk4P>(W, grid, s);
  if (sh.stack == kWalk4S) return enqueue_pass<kWalk4S>(W, grid, s);
  if (sh.stack == kWalk4) return enqueue_pass<kWalk4>(W, grid, s);
  if (sh.stack == 32) return enqueue_pass<32>(W, grid, s);
  return enqueue_pass<kStackDepth>(W, grid, s);
}

}  // namespace

cudaError_t render_pt_jobs(rx_context* c, const PtJob* jobs, int nj, const PtRun& run, double* film_sum,
                           double* film_sq, rx_render_stats* stats, PtShape* chosen, cudaStream_t s) {
  std::vector<SceneRec> recs(nj);
  uint64_t total = 0;
  uint32_t max_depth = 0, max_bvh_depth = 0;
  bool wide_ok = true;  // every scene's 4-wide BVH fits the 4-wide walk's stack
  // guiding: one network per distinct guiding state among the guided jobs
  std::vector<const GuideState*> net_state;
  for (int k = 0; k < nj; k++) {
    recs[k].S = jobs[k].ctx->scene;
    recs[k].P = make_pt_params(jobs[k].ctx, jobs[k].cam, jobs[k].opt);
    recs[k].path_begin = total;
    recs[k].pid_first = 0;
    recs[k].film_base = jobs[k].film_base;
    recs[k].paths = (uint64_t)recs[k].P.pixels * jobs[k].opt.spp;
    recs[k].net = -1;
    if (recs[k].paths >= (1ull << kLocalShift)) return cudaErrorInvalidValue;  // path ids keep 40 bits
    total += recs[k].paths;
    max_depth = std::max(max_depth, jobs[k].opt.max_depth);
    max_bvh_depth = std::max<uint32_t>(max_bvh_depth, (uint32_t)jobs[k].ctx->bvh.max_depth);
    const DevAccel& A = jobs[k].ctx->scene.accel;
    wide_ok = wide_ok && A.bvh4 && 3 * A.bvh4_depth + 1 <= 64;
    if ((jobs[k].opt.flags & RX_PT_GUIDED) && !jobs[k].opt.nee && guide_ready(jobs[k].ctx->guide)) {
      const GuideState* g = jobs[k].ctx->guide;
      auto it = std::find(net_state.begin(), net_state.end(), g);
      recs[k].net = (int)(it - net_state.begin());
      if (it == net_state.end()) net_state.push_back(g);
    }
  }
  const int nnet = (int)net_state.size();
  const bool guided = nnet > 0;
  // a pass slot index keeps 24 bits of the path id; interleaved passes add up to one slot
  // per scene to the pass size
  const uint32_t max_slots = (1u << 24) - (uint32_t)nj;
  uint32_t per_pass = run.paths_per_pass ? run.paths_per_pass : (1u << 22);
  per_pass = (uint32_t)std::min<uint64_t>(std::min<uint32_t>(per_pass, max_slots - (uint32_t)nj), total);
  if (per_pass == 0) return cudaSuccess;
  const uint64_t npasses = (total + per_pass - 1) / per_pass;
  // interleaved passes for guided renders (one schedule for all networks) and autotuned
  // ones (candidates timed on passes of the same mix; the passes after the tuning go
  // back to the concatenated layout)
  bool inter = guided || run.autotune;
  // per-scene quotas of a pass of about `size` paths: guided and untuned renders divide
  // every scene over the same number of passes; the queue-size candidates take their
  // share of `size` in proportion to the scenes' paths
  auto quotas = [&](uint32_t size, bool same_passes) {
    std::vector<uint32_t> q(nj);
    const uint64_t np = (total + size - 1) / size;
    for (int k = 0; k < nj; k++) {
      uint64_t v = same_passes ? (recs[k].paths + np - 1) / np
                               : (uint64_t)(((unsigned __int128)recs[k].paths * size + total - 1) / total);
      q[k] = (uint32_t)std::max<uint64_t>(recs[k].paths ? 1 : 0, std::min<uint64_t>(v, max_slots));
    }
    return q;
  };
  auto qsum = [](const std::vector<uint32_t>& q) {
    uint64_t s = 0;
    for (uint32_t v : q) s += v;
    return s;
  };
  const std::vector<uint32_t> q_default = quotas(per_pass, true);
  // queue-size candidates (untuned: the given size only)
  std::vector<uint32_t> sizes;
  if (run.autotune && !guided)
    for (uint32_t c : {1u << 20, 1u << 21, 1u << 22, 1u << 23})
      if (c <= max_slots - (uint32_t)nj && (uint64_t)c * 8 <= total) sizes.push_back(c);
  uint64_t slots64 = inter ? qsum(q_default) : per_pass;
  for (uint32_t c : sizes) slots64 = std::max<uint64_t>(slots64, qsum(quotas(c, false)));
  if (slots64 > max_slots) return cudaErrorInvalidValue;
  const uint32_t slots = (uint32_t)slots64;
  const int sms = c->trace_cfg.sms;

  std::vector<DevBuf> bufs;
  cudaError_t e;
  auto alloc = [&](size_t bytes) -> void* {
    bufs.emplace_back();
    if ((e = bufs.back().alloc(bytes)) != cudaSuccess) return nullptr;
    return bufs.back().p;
  };
  auto upload = [&](const void* src, size_t bytes) -> void* {
    void* p = alloc(bytes);
    if (p && (e = cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess) return nullptr;
    return p;
  };
  Wave W{};
  W.nr = nj;
  W.loops = max_depth + 1;
  W.film = film_sum;
  W.sq = film_sq;
  W.sms = sms;
  if (!(W.R = static_cast<const SceneRec*>(upload(recs.data(), sizeof(SceneRec) * nj)))) return e;
  PassState ps0{0, total, per_pass, 0, 0, inter ? 1u : 0u};
  if (!(W.ps = static_cast<PassState*>(upload(&ps0, sizeof ps0)))) return e;
  uint32_t* d_quota = nullptr;
  if (inter) {
    if (!(W.L.off = static_cast<uint32_t*>(alloc((size_t)(nj + 1) * 4)))) return e;
    if (!(W.L.taken = static_cast<uint64_t*>(alloc((size_t)nj * 8)))) return e;
    if (!(d_quota = static_cast<uint32_t*>(upload(q_default.data(), (size_t)nj * 4)))) return e;
    W.L.quota = d_quota;
    cudaMemsetAsync(W.L.taken, 0, (size_t)nj * 8, s);
  }
  if ((e = alloc_soa(W.A, bufs, slots)) != cudaSuccess) return e;
  if ((e = alloc_soa(W.B, bufs, slots)) != cudaSuccess) return e;
  if (!(W.hit = static_cast<int2*>(alloc(slots * sizeof(int2))))) return e;
  if (!(W.ctr = static_cast<unsigned long long*>(alloc(64 * sizeof(unsigned long long))))) return e;
  W.cnt = reinterpret_cast<unsigned*>(W.ctr + 8);
  cudaMemsetAsync(W.ctr, 0, 64 * sizeof(unsigned long long), s);
  if (run.bin && slots >= c->trace_cfg.bin_min && c->trace_cfg.bin_min) {
    if (!(W.keys = static_cast<uint32_t*>(alloc((size_t)slots * 4)))) return e;
    if (!(W.order = static_cast<uint32_t*>(alloc((size_t)slots * 4)))) return e;
    if (!(W.hist = static_cast<uint32_t*>(alloc((size_t)kRayBins * 4 + 4096)))) return e;
  }

  if (guided) {
    std::vector<guide::NetDev> nets(nnet);
    int steps = 0;
    uint32_t batch_max = 0;
    bool any_train = false;
    for (int j = 0; j < nnet; j++) {
      nets[j] = guide_net(net_state[j]);
      steps = std::max<int>(steps, (int)nets[j].steps_per_pass);
      batch_max = std::max(batch_max, nets[j].batch);
      any_train = any_train || (nets[j].train > 0 && nets[j].steps_per_pass > 0);
    }
    W.nnet = nnet;
    if (!(W.nets = static_cast<const guide::NetDev*>(upload(nets.data(), sizeof(guide::NetDev) * nnet)))) return e;
    std::vector<DevScene> sc(nj);
    for (int k = 0; k < nj; k++) sc[k] = recs[k].S;
    if (!(W.scenes = static_cast<const DevScene*>(upload(sc.data(), sizeof(DevScene) * nj)))) return e;
    if (!(W.lobes = static_cast<float*>(alloc((size_t)slots * guide::kLobeStride * sizeof(float))))) return e;
    if (nnet > 1) {
      if (!(W.ncount = static_cast<unsigned*>(alloc((size_t)nnet * 4)))) return e;
      if (!(W.cursor = static_cast<unsigned*>(alloc((size_t)nnet * 4)))) return e;
      if (!(W.seg = static_cast<uint32_t*>(alloc((size_t)(nnet + 1) * 4)))) return e;
      if (!(W.rows = static_cast<int*>(alloc(((size_t)slots + (size_t)nnet * guide::kGroupRows) * 4)))) return e;
      cudaMemsetAsync(W.ncount, 0, (size_t)nnet * 4, s);
    }
    if (any_train) {
      // raw records, then each network's region of the weighted records, sized by its
      // share of the pass's paths
      const uint32_t cap = (uint32_t)std::min<uint64_t>((uint64_t)slots * 4, 1u << 22);
      W.rec_cap = cap;
      if (!(W.recs = static_cast<float*>(alloc((size_t)cap * guide::kRec * sizeof(float))))) return e;
      if (!(W.train = static_cast<float*>(alloc((size_t)cap * guide::kRec * sizeof(float))))) return e;
      if (!(W.lpath = static_cast<float4*>(alloc((size_t)slots * sizeof(float4))))) return e;
      if (!(W.net_count = static_cast<unsigned*>(alloc((size_t)nnet * 4)))) return e;
      std::vector<uint64_t> share(nnet, 0);
      for (int k = 0; k < nj; k++)
        if (recs[k].net >= 0) share[recs[k].net] += q_default[k];
      uint64_t all = 0;
      for (uint64_t v : share) all += v;
      std::vector<uint32_t> rbase(nnet), rcap(nnet);
      std::vector<guide::RecSeg> segs(nnet);
      uint32_t acc = 0;
      for (int j = 0; j < nnet; j++) {
        rbase[j] = acc;
        rcap[j] = (uint32_t)((uint64_t)cap * share[j] / std::max<uint64_t>(all, 1));
        acc += rcap[j];
        segs[j] = guide::RecSeg{W.train + (size_t)rbase[j] * guide::kRec, W.net_count + j, rcap[j], nets[j].batch};
      }
      if (!(W.rbase = static_cast<const uint32_t*>(upload(rbase.data(), (size_t)nnet * 4)))) return e;
      if (!(W.rcap = static_cast<const uint32_t*>(upload(rcap.data(), (size_t)nnet * 4)))) return e;
      if (!(W.segs = static_cast<const guide::RecSeg*>(upload(segs.data(), sizeof(guide::RecSeg) * nnet)))) return e;
      W.steps = steps;
      W.batch_max = batch_max;
      cudaMemsetAsync(W.net_count, 0, (size_t)nnet * 4, s);
    }
    guide_prepare();  // kernel attributes set before any capture
  }

  // launch shapes: the context's default, or candidates timed on the first passes
  PtShape best{c->trace_cfg.pt_blocks_per_sm, wide_ok ? kWalk4P : (max_bvh_depth < 32 ? 32 : kStackDepth)};
  best.paths_per_pass = per_pass;
  std::vector<PtShape> cands;
  if (run.autotune) {
    // the walks that can win: the two 4-wide short-stack walks when every scene's 4-wide
    // tree fits (the binary walks and the all-local stack never did: each timing pass of
    // a candidate renders real samples at that candidate's speed), else the binary walks
    for (int bps : {4, 8, 16})
      for (int st : {kWalk4P, kWalk4S, 32, kStackDepth})
        if (st == kWalk4S || st == kWalk4P ? wide_ok : !wide_ok && st > (int)max_bvh_depth)
          cands.push_back(PtShape{bps, st, per_pass});
    if (npasses < 2 * cands.size() + 2) cands.clear();
  }

  Event e0, e1;
  if ((e = e0.create()) != cudaSuccess || (e = e1.create()) != cudaSuccess) return e;
  cudaEventRecord(e0, s);
  uint64_t pass = 0;
  // paths taken so far: per scene (interleaved passes, mirroring the device cursors) or
  // in all (concatenated)
  std::vector<uint64_t> taken(nj, 0);
  std::vector<uint32_t> q_now = q_default;
  uint64_t done_all = 0;
  auto account = [&]() -> uint64_t {  // one more pass: the paths it took
    uint64_t n = 0;
    if (inter) {
      for (int k = 0; k < nj; k++) {
        const uint32_t sh = pass_share(recs[k].paths, taken[k], q_now[k]);
        taken[k] += sh;
        n += sh;
      }
    } else {
      n = std::min<uint64_t>(per_pass, total - done_all);
    }
    done_all += n;
    return n;
  };
  auto set_quota = [&](const std::vector<uint32_t>& q) -> cudaError_t {
    q_now = q;
    return cudaMemcpyAsync(d_quota, q_now.data(), (size_t)nj * 4, cudaMemcpyHostToDevice, s);
  };
  // time budget: after queueing pass p, wait for pass p - 1 and stop if the wall time is
  // spent (pass p still completes)
  const auto t_start = std::chrono::steady_clock::now();
  Event pass_ev[2];
  if (run.time_budget_s > 0)
    for (auto& ev : pass_ev)
      if ((e = ev.create(cudaEventDisableTiming)) != cudaSuccess) return e;
  auto budget_spent = [&](uint64_t p) -> bool {
    if (run.time_budget_s <= 0) return false;
    cudaEventRecord(pass_ev[p & 1], s);
    if (p == 0) return false;
    cudaEventSynchronize(pass_ev[(p - 1) & 1]);
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count() >= run.time_budget_s;
  };
  // after queueing pass p: a due convergence snapshot (the film through pass p; one
  // scene only), then the budget; true = stop (e holds an error, if any)
  Snapshots snaps(c);
  const bool snap_on = nj == 1 && snaps.on();
  auto after_pass = [&](uint64_t p) -> bool {
    if (snap_on && snaps.due()) {
      const uint64_t done = done_all;
      const uint64_t npx = recs[0].P.pixels;
      e = snaps.take(film_sum, jobs[0].cam.width, jobs[0].cam.height, (double)done / (double)npx,
                     [&](size_t q) { return (double)(done / npx + (q < done % npx ? 1 : 0)); }, s);
      if (e != cudaSuccess) return true;
    }
    return budget_spent(p);
  };
  // candidates, each timed over two passes (ms per path); first the launch shapes at the
  // given pass size, then the pass sizes with the best shape
  if (!cands.empty()) {
    Event t0, t1;
    if ((e = t0.create()) != cudaSuccess || (e = t1.create()) != cudaSuccess) return e;
    auto time_passes = [&](const PtShape& sh, double& ms_per_path) -> cudaError_t {
      cudaEventRecord(t0, s);
      uint64_t n = 0;
      for (int r = 0; r < 2; r++) {
        cudaError_t err = enqueue_pass_shape(W, sh, sms, s);
        if (err != cudaSuccess) return err;
        n += account();
        pass++;
      }
      cudaEventRecord(t1, s);
      cudaError_t err = cudaEventSynchronize(t1);
      if (err != cudaSuccess) return err;
      float ms = 0;
      cudaEventElapsedTime(&ms, t0, t1);
      ms_per_path = n ? ms / (double)n : INFINITY;
      return cudaSuccess;
    };
    double best_t = INFINITY;
    for (const PtShape& sh : cands) {
      double tp;
      if ((e = time_passes(sh, tp)) != cudaSuccess) return e;
      if (tp < best_t) best_t = tp, best = sh;
    }
    // pass sizes, when their passes fit in what is left of the render
    uint64_t need = 0;
    for (uint32_t sz : sizes) need += 2 * qsum(quotas(sz, false));
    if (!sizes.empty() && done_all + need <= total) {
      best_t = INFINITY;
      PtShape bs = best;
      std::vector<uint32_t> best_q = q_now;
      for (uint32_t sz : sizes) {
        const std::vector<uint32_t> q = quotas(sz, false);
        if ((e = set_quota(q)) != cudaSuccess) return e;
        PtShape sh = best;
        sh.paths_per_pass = (uint32_t)qsum(q);
        double tp;
        if ((e = time_passes(sh, tp)) != cudaSuccess) return e;
        if (tp < best_t) best_t = tp, bs = sh, best_q = q;
      }
      best = bs;
      if ((e = set_quota(best_q)) != cudaSuccess) return e;
    }
  }
  if (chosen) *chosen = best;
  // Autotuned, unguided: the remaining passes take the scenes one after another again.
  // An interleaved pass touches every scene's tree and triangles (for a large batch far
  // more than L2 holds); a concatenated pass touches one or two scenes. Each scene
  // continues after the paths the tuning passes took from it.
  PassState ps_rest{};
  if (inter && !guided) {
    uint64_t begin = 0;
    for (int k = 0; k < nj; k++) {
      recs[k].pid_first = taken[k];
      recs[k].path_begin = begin;
      begin += recs[k].paths - taken[k];
    }
    per_pass = std::min<uint32_t>(best.paths_per_pass, slots);  // the path arrays hold `slots`
    ps_rest = PassState{0, begin, per_pass, 0, (uint32_t)pass, 0u};
    if ((e = cudaMemcpyAsync(const_cast<SceneRec*>(W.R), recs.data(), sizeof(SceneRec) * nj, cudaMemcpyHostToDevice,
                             s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(W.ps, &ps_rest, sizeof ps_rest, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return e;
    W.L = Layout{};
    inter = false;
  }

  // the remaining passes: one captured pass replayed, or enqueued one by one (a single
  // remaining pass is enqueued: capturing and instantiating a graph to replay it once
  // costs more than its launches, and the GPU would wait for the instantiation)
  auto left = [&]() { return done_all < total; };
  const bool several = total - done_all > (uint64_t)per_pass;
  if (run.use_graph && left() && several) {
    Graph graph;
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
    cudaError_t eq = enqueue_pass_shape(W, best, sms, s);
    e = cudaStreamEndCapture(s, &graph.g);
    if (eq != cudaSuccess) return eq;
    if (e != cudaSuccess) return e;
    if ((e = cudaGraphInstantiate(&graph.x, graph.g, 0)) != cudaSuccess) return e;
    while (left() && e == cudaSuccess) {
      e = cudaGraphLaunch(graph.x, s);
      account();
      if (e == cudaSuccess && after_pass(pass++)) break;
    }
    if (e != cudaSuccess) return e;
  } else {
    while (left()) {
      if ((e = enqueue_pass_shape(W, best, sms, s)) != cudaSuccess) return e;
      account();
      if (after_pass(pass++)) break;
    }
    if (e != cudaSuccess) return e;
  }
  cudaEventRecord(e1, s);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  if (stats) {
    unsigned long long h[2];
    cudaMemcpy(h, W.ctr, sizeof h, cudaMemcpyDeviceToHost);
    stats->extension_rays = h[0];
    stats->shadow_rays = h[1];
    stats->paths = done_all;
    stats->ms = ms;
  }
  return cudaSuccess;
}

cudaError_t render_pt(rx_context* c, const rx_camera& cam, const rx_pt_options& opt, double* film_sum,
                      double* film_sq, rx_render_stats* stats, cudaStream_t s) {
  PtJob job{c, cam, opt, 0};
  PtRun run{};
  run.paths_per_pass = opt.paths_per_pass;
  run.use_graph = true;
  run.time_budget_s = opt.time_budget_s > 0 ? opt.time_budget_s : 0;
  return render_pt_jobs(c, &job, 1, run, film_sum, film_sq, stats, nullptr, s);
}

}  // namespace rx
